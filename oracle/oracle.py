"""ctypes front-end of the oracle (oracle/rsa_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
cpu_baseline / reference legs of bench.py, always as the checker or the CPU
baseline.  The GPU library and its Python front-end never import this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "librsaoracle.so")
REF_BIN = os.path.join(HERE, "_ref", "ref_rsa")

_lib = None

_d = C.POINTER(C.c_double)
_u64 = C.POINTER(C.c_uint64)
_i64 = C.POINTER(C.c_int64)
_i32 = C.POINTER(C.c_int)
_u8 = C.POINTER(C.c_uint8)
_u32 = C.POINTER(C.c_uint32)


def build(force: bool = False) -> str:
    """Compiles the C restatement with make (gcc, -ffp-contract=off)."""
    src = os.path.join(HERE, "rsa_oracle.c")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True)
    return LIB_PATH


def build_ref(reference_root: str) -> str | None:
    """Compiles the reference driver into oracle/_ref when the reference checkout exists."""
    if not os.path.isdir(os.path.join(reference_root, "include")):
        return None
    subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={reference_root}"], check=True)
    return REF_BIN


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        L.ora_create.restype = C.c_void_p
        L.ora_create.argtypes = [C.c_int, _d, _d, C.c_double, C.c_int, _d, _u64, _i32, C.c_double, C.c_int]
        L.ora_reset_classes.argtypes = [C.c_void_p, C.c_int, _d, _u64, _i32, C.c_double]
        L.ora_create_uniform.restype = C.c_void_p
        L.ora_create_uniform.argtypes = [C.c_int, _d, _d, C.c_double, C.c_double, C.c_uint64, C.c_int, C.c_int]
        L.ora_destroy.argtypes = [C.c_void_p]
        L.ora_set_radius_table.argtypes = [C.c_void_p, _d, C.c_int]
        L.ora_count_from_fraction.restype = C.c_uint64
        L.ora_count_from_fraction.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double]
        L.ora_volume_sphere.restype = C.c_double
        L.ora_volume_sphere.argtypes = [C.c_int, C.c_double]
        L.ora_proceed.argtypes = [C.c_void_p, C.c_uint64]
        L.ora_begin.argtypes = [C.c_void_p, C.c_uint64]
        L.ora_gen_round.argtypes = [C.c_void_p, _u64, _u64, _i32]
        for name, rt in (("ora_cand_pos", _d), ("ora_cand_key", _u64), ("ora_cand_rad", _d), ("ora_cand_phase", _i32)):
            getattr(L, name).restype = rt
            getattr(L, name).argtypes = [C.c_void_p]
        L.ora_apply_round.argtypes = [C.c_void_p, C.c_uint64, _d, _u64, _d, _i32, C.c_uint64, C.c_int, _u8, _u64]
        L.ora_end_round.argtypes = [C.c_void_p, C.c_uint64, C.c_uint64, _i32]
        L.ora_refine.argtypes = [C.c_void_p]
        L.ora_voxel_count.restype = C.c_uint64
        L.ora_voxel_count.argtypes = [C.c_void_p]
        L.ora_voxel_export.argtypes = [C.c_void_p, _i64, _d]
        L.ora_voxel_level.argtypes = [C.c_void_p]
        L.ora_sphere_count.restype = C.c_uint64
        L.ora_sphere_count.argtypes = [C.c_void_p]
        L.ora_sphere_export.argtypes = [C.c_void_p, _d, _d, _i32]
        L.ora_sphere_import.argtypes = [C.c_void_p, C.c_uint64, _d, _d, _i32]
        L.ora_set_cap_exact.argtypes = [C.c_void_p, C.c_int]
        L.ora_ref_pivot.restype = C.c_int
        L.ora_ref_pivot.argtypes = [_u64, C.c_int64, C.c_int64, _d]
        L.ora_trace_len.restype = C.c_uint64
        L.ora_trace_len.argtypes = [C.c_void_p]
        L.ora_trace_export.argtypes = [C.c_void_p, _u64, _u64, _u64, _u8]
        L.ora_min_radius.restype = C.c_double
        L.ora_min_radius.argtypes = [C.c_void_p]
        L.ora_max_radius.restype = C.c_double
        L.ora_max_radius.argtypes = [C.c_void_p]
        L.ora_count_overlaps.restype = C.c_uint64
        L.ora_count_overlaps.argtypes = [C.c_int, _d, _d, C.c_uint64, _d, _d]
        L.ora_uncovered_after_refinement.restype = C.c_uint64
        L.ora_uncovered_after_refinement.argtypes = [C.c_int, _d, _d, C.c_uint64, _d, _d, C.c_double, C.c_double, C.c_int]
        L.ora_mt_seed_seq.argtypes = [C.c_void_p, _u32, C.c_int]
        L.ora_mt_next.restype = C.c_uint32
        L.ora_mt_next.argtypes = [C.c_void_p]
        L.ora_canonical.restype = C.c_double
        L.ora_canonical.argtypes = [C.c_void_p]
        L.ora_uniform_int.restype = C.c_uint32
        L.ora_uniform_int.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32]
        L.ora_poisson.restype = C.c_int
        L.ora_poisson.argtypes = [C.c_void_p, C.c_double]
        L.ora_philox4x32_10.argtypes = [_u32, _u32, _u32]
        _lib = L
    return _lib


def _p(a, t):
    return a.ctypes.data_as(t)


def volume_sphere(dim: int, r: float) -> float:
    return lib().ora_volume_sphere(dim, r)


def count_from_fraction(dim: int, r: float, phi: float, volume: float) -> int:
    return int(lib().ora_count_from_fraction(dim, r, phi, volume))


class Oracle:
    """One sampler instance on the box [inf, sup] (periodic)."""

    def __init__(self, dim, inf, sup, classes, domain_rad=None, exclusion=0.0, nbshots=6000,
                 volume=None, counts=None):
        """classes: list of (r, phi, phase) -- or (r, count, phase) when counts=True."""
        L = lib()
        self.dim = dim
        self.inf = np.ascontiguousarray(inf, dtype=np.float64)
        self.sup = np.ascontiguousarray(sup, dtype=np.float64)
        if volume is None:
            volume = float(np.prod(self.sup - self.inf))
        r = np.array([c[0] for c in classes], dtype=np.float64)
        if counts:
            n = np.array([int(c[1]) for c in classes], dtype=np.uint64)
        else:
            n = np.array([count_from_fraction(dim, c[0], c[1], volume) for c in classes], dtype=np.uint64)
        ph = np.array([int(c[2]) for c in classes], dtype=np.int32)
        if domain_rad is None:
            domain_rad = float(r.max())
        self._h = L.ora_create(dim, _p(self.inf, _d), _p(self.sup, _d), domain_rad, len(classes),
                               _p(r, _d), _p(n, _u64), _p(ph, _i32), exclusion, nbshots)
        if not self._h:
            raise RuntimeError("oracle: invalid configuration")

    @classmethod
    def uniform(cls, dim, inf, sup, r_min, r_max, count=10**16, phase=0, nbshots=6000):
        """A continuous radius law: each dart's radius r_min + (r_max - r_min) x, x ~ U[0, 1)
        (RadiusGenerator with a RandomRadiusGenerator, radius_generator.ixx:39-48)."""
        self = cls.__new__(cls)
        self.dim = dim
        self.inf = np.ascontiguousarray(inf, dtype=np.float64)
        self.sup = np.ascontiguousarray(sup, dtype=np.float64)
        self._h = lib().ora_create_uniform(dim, _p(self.inf, _d), _p(self.sup, _d), float(r_min), float(r_max),
                                           int(count), int(phase), int(nbshots))
        if not self._h:
            raise RuntimeError("oracle: invalid configuration")
        return self

    @classmethod
    def table(cls, dim, inf, sup, knots, count=10**16, phase=0, nbshots=6000):
        """A continuous radius law given by its transform's values at x = j / (len(knots) - 1), interpolated
        linearly (an arbitrary RandomRadiusGenerator transform, radius_generator.hxx:12-38)."""
        t = np.ascontiguousarray(knots, dtype=np.float64)
        self = cls.uniform(dim, inf, sup, float(t.min()), float(t.max()), count, phase, nbshots)
        if lib().ora_set_radius_table(self._h, _p(t, _d), len(t)) != 0:
            raise RuntimeError("oracle: invalid radius table")
        return self

    def reset(self, classes, volume=None, exclusion=0.0):
        """reset_radius_generator with classes (r, phi, phase) on the same domain and spheres."""
        if volume is None:
            volume = float(np.prod(self.sup - self.inf))
        r = np.array([c[0] for c in classes], dtype=np.float64)
        n = np.array([count_from_fraction(self.dim, c[0], c[1], volume) for c in classes], dtype=np.uint64)
        ph = np.array([int(c[2]) for c in classes], dtype=np.int32)
        if lib().ora_reset_classes(self._h, len(classes), _p(r, _d), _p(n, _u64), _p(ph, _i32), exclusion) != 0:
            raise RuntimeError("Incorrect maximal radius")

    def __del__(self):
        if getattr(self, "_h", None):
            lib().ora_destroy(self._h)
            self._h = None

    @property
    def r_min(self):
        return lib().ora_min_radius(self._h)

    @property
    def r_max(self):
        return lib().ora_max_radius(self._h)

    def proceed(self, seed):
        lib().ora_proceed(self._h, seed)

    def begin(self, seed):
        lib().ora_begin(self._h, seed)

    def gen_round(self):
        """Returns (status, candidates dict or None, max_new, may_outreach)."""
        n = C.c_uint64()
        mx = C.c_uint64()
        may = C.c_int()
        st = lib().ora_gen_round(self._h, C.byref(n), C.byref(mx), C.byref(may))
        if st != 0:
            return st, None, 0, 0
        k = n.value
        D = self.dim
        L = lib()
        cand = dict(
            pos=np.ctypeslib.as_array(L.ora_cand_pos(self._h), shape=(max(k, 1) * D,))[: k * D].reshape(k, D).copy(),
            key=np.ctypeslib.as_array(L.ora_cand_key(self._h), shape=(max(k, 1),))[:k].copy(),
            rad=np.ctypeslib.as_array(L.ora_cand_rad(self._h), shape=(max(k, 1),))[:k].copy(),
            phase=np.ctypeslib.as_array(L.ora_cand_phase(self._h), shape=(max(k, 1),))[:k].copy(),
        ) if k > 0 else dict(pos=np.zeros((0, D)), key=np.zeros(0, np.uint64), rad=np.zeros(0), phase=np.zeros(0, np.int32))
        return 0, cand, mx.value, may.value

    def apply_round(self, pos, key, rad, phase, max_new=2**63, may_outreach=0):
        pos = np.ascontiguousarray(pos, dtype=np.float64)
        key = np.ascontiguousarray(key, dtype=np.uint64)
        rad = np.ascontiguousarray(rad, dtype=np.float64)
        phase = np.ascontiguousarray(phase, dtype=np.int32)
        n = len(key)
        acc = np.zeros(max(n, 1), dtype=np.uint8)
        nn = C.c_uint64()
        lib().ora_apply_round(self._h, n, _p(pos, _d), _p(key, _u64), _p(rad, _d), _p(phase, _i32),
                              max_new, may_outreach, _p(acc, _u8), C.byref(nn))
        return acc[:n].astype(bool), nn.value

    def end_round(self, n_shots, n_new):
        ref = C.c_int()
        done = lib().ora_end_round(self._h, n_shots, n_new, C.byref(ref))
        return bool(done), bool(ref.value)

    def refine(self):
        lib().ora_refine(self._h)

    def voxels(self):
        n = lib().ora_voxel_count(self._h)
        coords = np.zeros((max(n, 1), self.dim), dtype=np.int64)
        ln = np.zeros(self.dim, dtype=np.float64)
        lib().ora_voxel_export(self._h, _p(coords, _i64), _p(ln, _d))
        return coords[:n], ln

    @property
    def voxel_level(self):
        return lib().ora_voxel_level(self._h)

    def spheres(self):
        n = lib().ora_sphere_count(self._h)
        pos = np.zeros((max(n, 1), self.dim))
        rad = np.zeros(max(n, 1))
        ph = np.zeros(max(n, 1), dtype=np.int32)
        lib().ora_sphere_export(self._h, _p(pos, _d), _p(rad, _d), _p(ph, _i32))
        return pos[:n], rad[:n], ph[:n]

    def import_spheres(self, pos, rad, phase=None):
        pos = np.ascontiguousarray(pos, dtype=np.float64)
        rad = np.ascontiguousarray(rad, dtype=np.float64)
        ph = np.ascontiguousarray(phase if phase is not None else np.zeros(len(rad)), dtype=np.int32)
        lib().ora_sphere_import(self._h, len(rad), _p(pos, _d), _p(rad, _d), _p(ph, _i32))

    def trace(self):
        n = lib().ora_trace_len(self._h)
        v = np.zeros(max(n, 1), np.uint64)
        s = np.zeros(max(n, 1), np.uint64)
        a = np.zeros(max(n, 1), np.uint64)
        r = np.zeros(max(n, 1), np.uint8)
        lib().ora_trace_export(self._h, _p(v, _u64), _p(s, _u64), _p(a, _u64), _p(r, _u8))
        return dict(voxels=v[:n], shots=s[:n], new=a[:n], refined=r[:n].astype(bool))


def count_overlaps(dim, inf, sup, pos, rad) -> int:
    inf = np.ascontiguousarray(inf, dtype=np.float64)
    sup = np.ascontiguousarray(sup, dtype=np.float64)
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    rad = np.ascontiguousarray(rad, dtype=np.float64)
    return int(lib().ora_count_overlaps(dim, _p(inf, _d), _p(sup, _d), len(rad), _p(pos, _d), _p(rad, _d)))


def uncovered_after_refinement(dim, inf, sup, pos, rad, r_max, r_min, max_levels=40) -> int:
    inf = np.ascontiguousarray(inf, dtype=np.float64)
    sup = np.ascontiguousarray(sup, dtype=np.float64)
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    rad = np.ascontiguousarray(rad, dtype=np.float64)
    return int(lib().ora_uncovered_after_refinement(dim, _p(inf, _d), _p(sup, _d), len(rad), _p(pos, _d),
                                                      _p(rad, _d), r_max, r_min, max_levels))


class MT19937:
    """std::mt19937 seeded with std::seed_seq{seeds...} (restated)."""

    def __init__(self, seeds):
        self._buf = C.create_string_buffer(624 * 4 + 16)
        s = np.ascontiguousarray(seeds, dtype=np.uint32)
        lib().ora_mt_seed_seq(self._buf, _p(s, _u32), len(s))

    def next(self):
        return lib().ora_mt_next(self._buf)

    def canonical(self):
        return lib().ora_canonical(self._buf)

    def uniform_int(self, lo, hi):
        return lib().ora_uniform_int(self._buf, lo, hi)

    def poisson(self, mean):
        return lib().ora_poisson(self._buf, mean)


def philox4x32_10(ctr, key):
    c = np.ascontiguousarray(ctr, dtype=np.uint32)
    k = np.ascontiguousarray(key, dtype=np.uint32)
    out = np.zeros(4, dtype=np.uint32)
    lib().ora_philox4x32_10(_p(c, _u32), _p(k, _u32), _p(out, _u32))
    return out


def read_ref_spheres(path):
    """Reads the binary sphere file written by oracle/_ref/ref_rsa."""
    with open(path, "rb") as f:
        dim = int(np.frombuffer(f.read(4), np.int32)[0])
        n = int(np.frombuffer(f.read(8), np.int64)[0])
        rec = np.dtype([("c", np.float64, (dim,)), ("r", np.float64), ("p", np.int32)])
        arr = np.frombuffer(f.read(n * rec.itemsize), dtype=rec)
    return arr["c"].copy(), arr["r"].copy(), arr["p"].copy()
