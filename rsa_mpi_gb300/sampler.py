"""Python classes over the C ABI: Domain, RadiusGenerator, Algo.

They own the C handles and mirror the reference's user_interface classes
(include/user_interface.hxx:13-110): an Algo keeps a reference to its Domain
(which it must not outlive) and a copy of the radius generator; creating an Algo
clears the Domain's spheres.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import check, lib, ptr


class Domain:
    """Periodic box [inf, sup] in dimension len(inf) (rsa_domain, include/rsa_domain.hxx:18-94)."""

    def __init__(self, inf, sup, rad_max: float):
        inf = np.ascontiguousarray(inf, dtype=np.float64)
        sup = np.ascontiguousarray(sup, dtype=np.float64)
        if inf.shape != sup.shape or inf.ndim != 1:
            raise RuntimeError("inf and sup must be vectors of the same size")
        self.dim = int(inf.shape[0])
        self.inf = inf
        self.sup = sup
        self.rad_max = float(rad_max)
        h = C.c_void_p()
        check(lib().rsagpu_domain_create(self.dim, ptr(inf, _lib._d), ptr(sup, _lib._d), self.rad_max, C.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            lib().rsagpu_domain_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def total_volume(self) -> float:
        v = C.c_double()
        check(lib().rsagpu_domain_total_volume(self._h, C.byref(v)))
        return v.value

    def spheres_volume(self) -> float:
        v = C.c_double()
        check(lib().rsagpu_domain_spheres_volume(self._h, C.byref(v)))
        return v.value

    def count(self) -> int:
        v = C.c_uint64()
        check(lib().rsagpu_domain_count(self._h, C.byref(v)))
        return v.value

    def arrays(self):
        """(centers [n, dim], radii [n], phases [n]) of the placed spheres, in cell order."""
        n = C.c_uint64()
        check(lib().rsagpu_domain_extract(self._h, None, None, None, 0, C.byref(n)))
        k = n.value
        pos = np.zeros((max(k, 1), self.dim), dtype=np.float64)
        rad = np.zeros(max(k, 1), dtype=np.float64)
        ph = np.zeros(max(k, 1), dtype=np.int32)
        check(lib().rsagpu_domain_extract(self._h, ptr(pos, _lib._d), ptr(rad, _lib._d), ptr(ph, _lib._i32),
                                          k, C.byref(n)))
        return pos[:k], rad[:k], ph[:k]

    def check(self):
        """(overlapping pairs, misplaced spheres), exact FP64 on the device."""
        a = C.c_uint64()
        b = C.c_uint64()
        check(lib().rsagpu_domain_check(self._h, C.byref(a), C.byref(b)))
        return a.value, b.value


class RadiusGenerator:
    """Radius classes (sac_de_billes::RadiusGenerator, include/radius_generator.hxx:46-105)."""

    def __init__(self, dim: int, classes, volume: float | None = None, exclusion: float = 0.0):
        """classes = [(r, N, phase), ...] when volume is None, else [(r, phi, phase), ...]."""
        self.dim = dim
        r = np.ascontiguousarray([float(c[0]) for c in classes], dtype=np.float64)
        ph = np.ascontiguousarray([int(c[2]) for c in classes], dtype=np.int32)
        h = C.c_void_p()
        if volume is None:
            n = np.ascontiguousarray([int(c[1]) for c in classes], dtype=np.uint64)
            check(lib().rsagpu_radgen_create_counts(dim, ptr(r, _lib._d), ptr(n, _lib._u64), ptr(ph, _lib._i32),
                                                    len(classes), float(exclusion), C.byref(h)))
        else:
            phi = np.ascontiguousarray([float(c[1]) for c in classes], dtype=np.float64)
            check(lib().rsagpu_radgen_create_fractions(dim, ptr(r, _lib._d), ptr(phi, _lib._d), ptr(ph, _lib._i32),
                                                       len(classes), float(volume), float(exclusion), C.byref(h)))
        self._h = h

    @classmethod
    def uniform(cls, dim: int, r_min: float, r_max: float, count: int = 10**16, phase: int = 0):
        """Continuous radius law: each sphere's radius r_min + (r_max - r_min) x, x uniform in [0, 1)
        (RadiusGenerator with a RandomRadiusGenerator, include/radius_generator.hxx:12-38); count spheres
        wanted, 10^16 running to maximality."""
        self = cls.__new__(cls)
        self.dim = dim
        h = C.c_void_p()
        check(lib().rsagpu_radgen_create_uniform(dim, float(r_min), float(r_max), int(count), int(phase), C.byref(h)))
        self._h = h
        return self

    @classmethod
    def transform(cls, dim: int, f, count: int = 10**16, phase: int = 0, knots: int = 4097):
        """Continuous radius law with any transform f of x uniform in [0, 1) (the reference's
        RandomRadiusGenerator, include/radius_generator.hxx:12-38): f is tabulated at `knots` points
        x = j / (knots - 1) and the darts interpolate it linearly."""
        x = np.arange(knots, dtype=np.float64) / (knots - 1)
        t = np.ascontiguousarray([float(f(v)) for v in x], dtype=np.float64)
        self = cls.__new__(cls)
        self.dim = dim
        h = C.c_void_p()
        check(lib().rsagpu_radgen_create_table(dim, ptr(t, _lib._d), len(t), int(count), int(phase), C.byref(h)))
        self._h = h
        return self

    def __del__(self):
        if getattr(self, "_h", None):
            try:
                lib().rsagpu_radgen_destroy(self._h)
            except Exception:
                pass
            self._h = None

    @property
    def max_radius(self) -> float:
        v = C.c_double()
        check(lib().rsagpu_radgen_max_radius(self._h, C.byref(v)))
        return v.value

    @property
    def min_radius(self) -> float:
        v = C.c_double()
        check(lib().rsagpu_radgen_min_radius(self._h, C.byref(v)))
        return v.value


class Algo:
    """The sampler (algorithm::rsa_algo, include/operator_algorithm.hxx:18-109)."""

    def __init__(self, domain: Domain, radgen: RadiusGenerator, nbshots: int = 6000):
        h = C.c_void_p()
        check(lib().rsagpu_algo_create(domain._h, radgen._h, int(nbshots), C.byref(h)))
        self._h = h
        self.domain = domain  # the domain must outlive the algo
        self.dim = domain.dim

    def close(self):
        if getattr(self, "_h", None):
            lib().rsagpu_algo_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_form(self, form: int = _lib.RSAGPU_FORM_FP64, schedule: int = _lib.RSAGPU_SCHEDULE_HEURISTIC):
        check(lib().rsagpu_algo_set_form(self._h, form, schedule))

    def set_cap_rule(self, rule: int):
        check(lib().rsagpu_algo_set_cap_rule(self._h, rule))

    def set_inherit(self, on: bool = True):
        """Sphere lists handed from voxels to their children in the FP32 3D mask pass; off (the default) walks
        every voxel's whole neighbourhood.  Either way the decisions are the same."""
        check(lib().rsagpu_algo_set_inherit(self._h, 1 if on else 0))

    def set_schedule(self, factor=0.25, min_darts=4096, max_darts=1 << 26, miss_threshold=0.99):
        check(lib().rsagpu_algo_set_schedule_params(self._h, float(factor), int(min_darts), int(max_darts),
                                                    float(miss_threshold)))

    def set_mlp(self, weights_bf16: np.ndarray):
        w = np.ascontiguousarray(weights_bf16, dtype=np.uint16)
        check(lib().rsagpu_algo_set_mlp(self._h, ptr(w, _lib._u16), len(w)))

    def set_timing(self, on: bool = True):
        check(lib().rsagpu_algo_set_timing(self._h, 1 if on else 0))

    def kernel_profile(self):
        """(ms, algorithmic bytes, parent voxels) per refine-mask launch of the last proceed()."""
        n = C.c_uint64()
        check(lib().rsagpu_algo_kernel_profile(self._h, None, None, None, 0, C.byref(n)))
        k = n.value
        ms = np.zeros(max(k, 1))
        by = np.zeros(max(k, 1))
        vx = np.zeros(max(k, 1))
        check(lib().rsagpu_algo_kernel_profile(self._h, ptr(ms, _lib._d), ptr(by, _lib._d), ptr(vx, _lib._d), k,
                                               C.byref(n)))
        return ms[:k], by[:k], vx[:k]

    def proceed(self, seed: int):
        check(lib().rsagpu_algo_proceed(self._h, int(seed)))

    def reset_radius_generator(self, radgen: RadiusGenerator):
        check(lib().rsagpu_algo_reset_radgen(self._h, radgen._h))

    def stats(self) -> dict:
        s = _lib.Stats()
        check(lib().rsagpu_algo_stats(self._h, C.byref(s)))
        return s.as_dict()

    def trace(self) -> dict:
        n = C.c_uint64()
        check(lib().rsagpu_algo_trace(self._h, None, None, None, None, None, 0, C.byref(n)))
        k = n.value
        v = np.zeros(max(k, 1), np.uint64)
        d = np.zeros(max(k, 1), np.uint64)
        a = np.zeros(max(k, 1), np.uint64)
        r = np.zeros(max(k, 1), np.uint8)
        lv = np.zeros(max(k, 1), np.int32)
        check(lib().rsagpu_algo_trace(self._h, ptr(v, _lib._u64), ptr(d, _lib._u64), ptr(a, _lib._u64),
                                      ptr(r, _lib._u8), lv.ctypes.data_as(C.POINTER(C.c_int32)), k, C.byref(n)))
        return dict(voxels=v[:k], darts=d[:k], accepted=a[:k], refined=r[:k].astype(bool), level=lv[:k])

    # ---- replay seam ----
    def begin(self):
        check(lib().rsagpu_algo_begin(self._h))

    def replay_round(self, pos, key, rad, phase=None, max_new=2**63, may_outreach=False):
        pos = np.ascontiguousarray(pos, dtype=np.float64)
        key = np.ascontiguousarray(key, dtype=np.uint64)
        rad = np.ascontiguousarray(rad, dtype=np.float64)
        n = len(key)
        ph = np.ascontiguousarray(phase if phase is not None else np.zeros(n), dtype=np.int32)
        acc = np.zeros(max(n, 1), dtype=np.uint8)
        nn = C.c_uint64()
        check(lib().rsagpu_algo_replay_round(self._h, n, ptr(pos, _lib._d), ptr(key, _lib._u64), ptr(rad, _lib._d),
                                             ptr(ph, _lib._i32), int(max_new), 1 if may_outreach else 0,
                                             ptr(acc, _lib._u8), C.byref(nn)))
        return acc[:n].astype(bool), nn.value

    def end_round(self, n_shots: int, n_new: int):
        r = C.c_int()
        d = C.c_int()
        check(lib().rsagpu_algo_end_round(self._h, int(n_shots), int(n_new), C.byref(r), C.byref(d)))
        return bool(d.value), bool(r.value)

    def refine(self):
        check(lib().rsagpu_algo_refine(self._h))

    def voxels(self):
        n = C.c_uint64()
        lv = C.c_int32()
        ln = np.zeros(self.dim)
        check(lib().rsagpu_algo_voxels(self._h, None, 0, C.byref(n), C.byref(lv), ptr(ln, _lib._d)))
        k = n.value
        coords = np.zeros((max(k, 1), self.dim), dtype=np.int64)
        check(lib().rsagpu_algo_voxels(self._h, ptr(coords, _lib._i64), k, C.byref(n), C.byref(lv), ptr(ln, _lib._d)))
        return coords[:k], ln, lv.value

    def draw_darts(self, seed: int, round_: int, n: int):
        pos = np.zeros((max(n, 1), self.dim))
        key = np.zeros(max(n, 1), np.uint64)
        vidx = np.zeros(max(n, 1), np.uint64)
        check(lib().rsagpu_algo_draw_darts(self._h, int(seed), int(round_), int(n), ptr(pos, _lib._d),
                                           ptr(key, _lib._u64), ptr(vidx, _lib._u64)))
        return pos[:n], key[:n], vidx[:n]


def kernel_launches() -> int:
    return int(lib().rsagpu_kernel_launches())


def batch_run(instances, form: int = _lib.RSAGPU_FORM_FP32_GUARD, max_bytes: int = 0, autotune: bool = True):
    """Runs independent one-radius instances to maximality in batched launches (rsagpu_batch_run).

    instances: sequence of (dim, sup, radius, seed), the box being [0, sup].  Returns a dict with
    per-instance ``counts``, ``checksums`` (see sphere_checksum) and ``seconds`` (time to maximality),
    and the run's ``stats``.
    """
    n = len(instances)
    arr = (_lib.InstanceDesc * max(n, 1))()
    for i, (dim, sup, radius, seed) in enumerate(instances):
        arr[i].dim = int(dim)
        for d in range(min(int(dim), _lib.MAX_DIM, len(sup))):
            arr[i].sup[d] = float(sup[d])
        arr[i].radius = float(radius)
        arr[i].seed = int(seed)
    counts = np.zeros(max(n, 1), np.uint64)
    sums = np.zeros(max(n, 1), np.uint64)
    secs = np.zeros(max(n, 1))
    st = _lib.BatchStats()
    check(lib().rsagpu_batch_run(arr, n, int(form), int(max_bytes), 1 if autotune else 0, ptr(counts, _lib._u64),
                                 ptr(sums, _lib._u64), ptr(secs, _lib._d), C.byref(st)))
    stats = {k: getattr(st, k) for k, _ in _lib.BatchStats._fields_ if k != "block"}
    stats["block"] = {d: list(st.block[d]) for d in range(2, _lib.MAX_DIM + 1) if any(st.block[d])}
    return {"counts": counts[:n], "checksums": sums[:n], "seconds": secs[:n], "stats": stats}


def expected_spheres(instance) -> float:
    """The work estimate of one batched instance (dim, sup, radius, seed): its box volume over the volume of
    one sphere, proportional to the spheres of its maximal packing."""
    dim, sup, radius, _ = instance
    vol = 1.0
    for d in range(int(dim)):
        vol *= float(sup[d])
    return vol / _ball_volume(int(dim), float(radius))


def _ball_volume(dim: int, r: float) -> float:
    import math
    return math.pi ** (dim / 2) / math.gamma(dim / 2 + 1) * r ** dim


def partition_instances(instances, world: int):
    """Splits independent instances over `world` ranks, balanced by expected_spheres: the largest instance
    first to the rank with the least work so far (ties to the lower rank).  Returns one sorted index list per
    rank; the lists are disjoint and together hold every instance.  Deterministic, so every rank computes the
    same split with no exchange.  (The reference decomposes one domain over MPI ranks with ghost layers,
    rsa_ghost_area / operator_ghost; independent instances need no exchange at all.)"""
    import heapq
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(instances)), key=lambda i: (-expected_spheres(instances[i]), i))
    heap = [(0.0, r) for r in range(world)]
    parts = [[] for _ in range(world)]
    for i in order:
        load, r = heapq.heappop(heap)
        parts[r].append(i)
        heapq.heappush(heap, (load + expected_spheres(instances[i]), r))
    return [sorted(p) for p in parts]


def _mix64(z: np.ndarray) -> np.ndarray:
    z = z ^ (z >> np.uint64(30))
    z = z * np.uint64(0xBF58476D1CE4E5B9)
    z = z ^ (z >> np.uint64(27))
    z = z * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def sphere_checksum(centers: np.ndarray) -> int:
    """The order-free checksum rsagpu_batch_run reports for a set of centres (n x dim, FP64)."""
    c = np.ascontiguousarray(centers, dtype=np.float64)
    if c.size == 0:
        return 0
    bits = c.view(np.uint64).reshape(c.shape)
    with np.errstate(over="ignore"):
        h = np.full(c.shape[0], 0x9E3779B97F4A7C15, dtype=np.uint64)
        for d in range(c.shape[1]):
            h = _mix64(h ^ bits[:, d])
        return int(h.sum(dtype=np.uint64))
