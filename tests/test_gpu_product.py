"""The product path (Philox darts, GPU schedule) on the GPU: validity, maximality, statistics, and the
dart kernel against its formula; plus replay edge cases (ties, exact contact, periodic wrap, empty)."""
import numpy as np
import pytest

from oracle import oracle as O
from rsa_mpi_gb300 import _lib
from rsa_mpi_gb300.sampler import Algo, Domain, RadiusGenerator
from gpu_helpers import INDEX, sort_spheres, sort_voxels

pytestmark = pytest.mark.gpu


def run_product(dim, L, r, seed, **sched):
    rg = RadiusGenerator(dim, [(r, 1.0, 0)], volume=float(np.prod(L)))
    dom = Domain([0.0] * dim, L, r)
    algo = Algo(dom, rg, 6000)
    if sched:
        algo.set_schedule(**sched)
    algo.proceed(seed)
    return dom, algo


@pytest.mark.parametrize("dim,L,r,phi_ref,tol", [
    (2, [1.0, 1.0], 0.005, 0.547187, 0.006),      # config 1 (reference: 6,967 discs, 0.547187)
    (3, [1.0, 1.0, 1.0], 0.02, 0.385201, 0.008),  # reference: 11,495 spheres, 0.38520
    (2, [1.3, 0.7], 0.02, 0.500142 / (1.3 * 0.7), 0.03),  # reference n2d_rect_s7: 398 discs
])
def test_product_run_is_valid_maximal_and_matches_fraction(dim, L, r, phi_ref, tol):
    dom, algo = run_product(dim, L, r, 7)
    st = algo.stats()
    assert st["maximal"] == 1
    pos, rad, ph = dom.arrays()
    assert dom.check() == (0, 0)
    inf = [0.0] * dim
    assert O.count_overlaps(dim, inf, L, pos, rad) == 0
    assert O.uncovered_after_refinement(dim, inf, L, pos, rad, r, r, 40) == 0
    phi = len(rad) * O.volume_sphere(dim, r) / float(np.prod(L))
    assert abs(dom.spheres_volume() / float(np.prod(L)) - phi) < 1e-9
    assert abs(phi - phi_ref) < tol, (phi, phi_ref)


@pytest.mark.parametrize("dim,L,r", [(2, [1.0, 1.0], 0.005), (3, [1.0, 1.0, 1.0], 0.01), (3, [0.9, 1.1, 1.0], 0.013)])
def test_fp32_guard_form_gives_the_fp64_form_output(dim, L, r):
    """The FP32 screen decides only outside the guard band and retests the rest in FP64: same spheres."""
    out = []
    for form in (_lib.RSAGPU_FORM_FP64, _lib.RSAGPU_FORM_FP32_GUARD):
        rg = RadiusGenerator(dim, [(r, 1.0, 0)], volume=float(np.prod(L)))
        dom = Domain([0.0] * dim, L, r)
        algo = Algo(dom, rg, 6000)
        algo.set_form(form)
        algo.proceed(11)
        out.append((dom.arrays()[0], algo.stats()))
    np.testing.assert_array_equal(out[0][0], out[1][0])
    assert out[0][1]["retests"] == 0 and out[1][1]["retests"] > 0
    assert out[1][1]["maximal"] == 1


@pytest.mark.parametrize("dim,L,classes", [
    (4, [1.0, 1.0, 1.0, 1.0], [(0.08, 1.0, 0)]),
    (5, [1.0] * 5, [(0.12, 1.0, 0)]),
    (2, [1.0, 0.8], [(0.02, 0.3, 0), (0.01, 0.1, 1)]),
    (3, [1.0, 1.0, 1.0], [(0.02, 0.2, 0), (0.01, 0.1, 1), (0.005, 0.02, 2)]),
])
def test_fp32_guard_form_matches_fp64_in_higher_dimensions_and_with_classes(dim, L, classes):
    """The FP32 form's fixed-point maps, lazy dart positions and point-trimmed walks in D = 4, 5 and with
    several radius classes (count caps included): the same spheres as the plain FP64 form, and no overlap."""
    out = []
    for form in (_lib.RSAGPU_FORM_FP64, _lib.RSAGPU_FORM_FP32_GUARD):
        rg = RadiusGenerator(dim, classes, volume=float(np.prod(L)))
        dom = Domain([0.0] * dim, L, rg.max_radius)
        algo = Algo(dom, rg, 6000)
        algo.set_form(form)
        algo.proceed(5)
        pos, rad, ph = dom.arrays()
        out.append((pos, rad, ph, algo.stats()))
        assert dom.check() == (0, 0)
    np.testing.assert_array_equal(out[0][0], out[1][0])
    np.testing.assert_array_equal(out[0][1], out[1][1])
    np.testing.assert_array_equal(out[0][2], out[1][2])
    assert O.count_overlaps(dim, [0.0] * dim, L, out[1][0], out[1][1]) == 0
    if len(classes) == 1:
        assert out[1][3]["maximal"] == 1
        # maximality re-certified by the oracle's own subdivision (all 2^D children)
        r = classes[0][0]
        assert O.uncovered_after_refinement(dim, [0.0] * dim, L, out[1][0], out[1][1], r, r, 40) == 0


@pytest.mark.parametrize("dim,L,r", [(2, [1.0, 1.0], 0.01), (3, [1.0, 0.9, 1.1], 0.02), (5, [1.0] * 5, 0.15)])
def test_extract_into_pinned_host_buffers(dim, L, r):
    """rsagpu_domain_extract into pinned host buffers (written by the kernel across the link, no device staging)
    gives the arrays of the staged path into ordinary (pageable) buffers, bit for bit."""
    import ctypes as C
    torch = pytest.importorskip("torch")
    dom, algo = run_product(dim, L, r, 3)
    pos, rad, ph = dom.arrays()
    n = len(rad)
    P = torch.empty((n + 7, dim), dtype=torch.float64, pin_memory=True).numpy()
    R = torch.empty(n + 7, dtype=torch.float64, pin_memory=True).numpy()
    H = torch.empty(n + 7, dtype=torch.int32, pin_memory=True).numpy()
    k = C.c_uint64()
    L_ = _lib.lib()
    for out in ((P, R, H), (P, None, None), (None, R, H)):
        for a in out:
            if a is not None:
                a.fill(-1)
        args = [_lib.ptr(out[0], _lib._d) if out[0] is not None else None,
                _lib.ptr(out[1], _lib._d) if out[1] is not None else None,
                _lib.ptr(out[2], _lib._i32) if out[2] is not None else None]
        _lib.check(L_.rsagpu_domain_extract(dom._h, *args, n + 7, C.byref(k)))
        assert k.value == n
        if out[0] is not None:
            np.testing.assert_array_equal(out[0][:n], pos)
            assert np.all(out[0][n:] == -1)  # nothing written past the spheres
        if out[1] is not None:
            np.testing.assert_array_equal(out[1][:n], rad)
            np.testing.assert_array_equal(out[2][:n], ph)
    algo.close()
    dom.close()


def test_class_overshoot_ends_the_class():
    """A capped round under the reference's pivot rule can keep more spheres than its class still wants (here the
    first round of the 0.004 class, in some of the seeds).  The product loop then ends the class and draws the
    next ones; the reference's size_t count would wrap and throw the first radius until no voxel is left.  Scaled
    config 3 (box side 0.25: 1/64 of its volume), both forms, four seeds."""
    classes = [(0.004, 0.20, 0), (0.002, 0.10, 0), (0.001, 0.05, 0)]
    side = 0.25
    targets = [int(side ** 3 * f / O.volume_sphere(3, r)) for r, f, _ in classes]
    overshoots = 0
    for seed in (1, 2, 3, 4):
        out = []
        for form in (_lib.RSAGPU_FORM_FP64, _lib.RSAGPU_FORM_FP32_GUARD):
            rg = RadiusGenerator(3, classes, volume=side ** 3)
            dom = Domain([0.0] * 3, [side] * 3, rg.max_radius)
            algo = Algo(dom, rg, 6000)
            algo.set_form(form)
            algo.proceed(seed)
            pos, rad, _ = dom.arrays()
            assert dom.check() == (0, 0)
            out.append((pos, rad))
            algo.close()
            dom.close()
        np.testing.assert_array_equal(out[0][0], out[1][0])
        rad = out[1][1]
        per_class = [int(np.count_nonzero(rad == r)) for r, _, _ in classes]
        assert per_class[0] >= targets[0] and per_class[1:] == targets[1:], (seed, per_class, targets)
        assert per_class[0] <= targets[0] * 1.02
        overshoots += per_class[0] > targets[0]
        assert O.count_overlaps(3, [0.0] * 3, [side] * 3, out[1][0], rad) == 0
    assert overshoots >= 1  # the case this test is about occurred


@pytest.mark.parametrize("L,r,seed", [([1.0] * 3, 0.01, 3), ([0.6, 0.5, 0.4], 0.006, 4), ([1.0] * 3, 0.005, 5)])
def test_inherited_sphere_lists_give_the_full_walk_result(L, r, seed):
    """FP32 form, 3D: the mask pass hands each surviving voxel's nearby spheres to its children, which test those
    plus the spheres placed since instead of walking their whole neighbourhood.  Against every voxel walking its
    whole neighbourhood: the same voxel count after every refinement, the same spheres, maximal."""
    out = []
    for on in (True, False):
        rg = RadiusGenerator(3, [(r, 1.0, 0)], volume=float(np.prod(L)))
        dom = Domain([0.0] * 3, L, r)
        algo = Algo(dom, rg, 6000)
        algo.set_form(_lib.RSAGPU_FORM_FP32_GUARD)
        algo.set_inherit(on)
        algo.proceed(seed)
        st = algo.stats()
        assert st["maximal"] == 1 and dom.check() == (0, 0)
        out.append((dom.arrays()[0], algo.trace()["voxels"], st))
    assert out[0][2]["final_level"] >= 4
    np.testing.assert_array_equal(out[0][1], out[1][1])
    np.testing.assert_array_equal(out[0][0], out[1][0])


@pytest.mark.parametrize("dim,r", [(6, 0.3), (7, 0.4)])
def test_six_and_seven_dimensions(dim, r):
    """D = 6 and 7 (64 and 128 children per voxel, child masks of several words): both forms run to an empty
    voxel list, give the same spheres, and the oracle's exact FP64 check finds no overlap."""
    L = [1.0] * dim
    out = []
    for form in (_lib.RSAGPU_FORM_FP64, _lib.RSAGPU_FORM_FP32_GUARD):
        rg = RadiusGenerator(dim, [(r, 1.0, 0)], volume=1.0)
        dom = Domain([0.0] * dim, L, r)
        algo = Algo(dom, rg, 6000)
        algo.set_form(form)
        algo.proceed(9)
        st = algo.stats()
        assert st["maximal"] == 1 and st["final_level"] > 0
        pos, rad, ph = dom.arrays()
        assert dom.check() == (0, 0)
        out.append(pos)
    np.testing.assert_array_equal(out[0], out[1])
    assert len(out[0]) >= 5
    assert O.count_overlaps(dim, [0.0] * dim, L, out[1], np.full(len(out[1]), r)) == 0


@pytest.mark.parametrize("dim,L,r0,r1,phi_ref", [
    (2, [1.0, 1.0], 0.02, 0.025, 0.585),     # reference u2d_r0.02-0.025_s7: 0.58495
    (3, [1.0, 1.0, 1.0], 0.05, 0.055, 0.40),  # reference u3d_r0.05-0.055_s0: 0.40099
])
def test_continuous_radius_law_product_path(dim, L, r0, r1, phi_ref):
    """Per-dart radii (the reference's RandomRadiusGenerator with a uniform transform): radii in [r0, r1), all
    distinct, no overlap, no voxel left uncovered for r0, the FP32 form equal to the FP64 form, and the packing
    fraction of the reference's run within sampling noise."""
    out = []
    for form in (_lib.RSAGPU_FORM_FP64, _lib.RSAGPU_FORM_FP32_GUARD):
        fr = []
        for seed in range(6):
            rg = RadiusGenerator.uniform(dim, r0, r1)
            dom = Domain([0.0] * dim, L, rg.max_radius)
            algo = Algo(dom, rg, 6000)
            algo.set_form(form)
            algo.proceed(40 + seed)
            assert algo.stats()["maximal"] == 1
            pos, rad, ph = dom.arrays()
            assert dom.check() == (0, 0)
            if seed == 0:
                out.append((pos, rad))
                assert np.all(rad >= r0) and np.all(rad < r1) and len(np.unique(rad)) == len(rad)
                assert O.count_overlaps(dim, [0.0] * dim, L, pos, rad) == 0
                assert O.uncovered_after_refinement(dim, [0.0] * dim, L, pos, rad, r1, r0, 40) == 0
            fr.append(sum(O.volume_sphere(dim, x) for x in rad) / float(np.prod(L)))
        assert abs(np.mean(fr) - phi_ref) < 0.02, fr
    np.testing.assert_array_equal(out[0][0], out[1][0])
    np.testing.assert_array_equal(out[0][1], out[1][1])


@pytest.mark.parametrize("dim,L,radii", [
    (2, [1.0, 1.0], (0.02, 0.012, 0.006)),
    (3, [1.0, 1.0, 1.0], (0.05, 0.03)),
])
def test_reiteration_product_path(dim, L, radii):
    """reset_radius_generator to smaller radii on the same domain, proceeding after each reset: the grid is
    rebuilt for the new radius, the old spheres stay, the result is maximal for the last radius, no overlap,
    and the FP32 form places the same spheres as the FP64 form."""
    out = []
    vol = float(np.prod(L))
    for form in (_lib.RSAGPU_FORM_FP64, _lib.RSAGPU_FORM_FP32_GUARD):
        dom = Domain([0.0] * dim, L, radii[0])
        algo = Algo(dom, RadiusGenerator(dim, [(radii[0], 1.0, 0)], volume=vol), 6000)
        algo.set_form(form)
        n_prev = 0
        for i, r in enumerate(radii):
            if i:
                algo.reset_radius_generator(RadiusGenerator(dim, [(r, 1.0, 0)], volume=vol))
            algo.proceed(11 + i)
            assert algo.stats()["maximal"] == 1
            pos, rad, ph = dom.arrays()
            assert len(rad) > n_prev and np.count_nonzero(rad == r) == len(rad) - n_prev
            n_prev = len(rad)
            assert dom.check() == (0, 0)
        assert O.count_overlaps(dim, [0.0] * dim, L, pos, rad) == 0
        assert O.uncovered_after_refinement(dim, [0.0] * dim, L, pos, rad, radii[0], radii[-1], 40) == 0
        out.append(sort_spheres(pos, rad, ph))
    for a, b in zip(*out):
        np.testing.assert_array_equal(a, b)


def test_product_runs_are_deterministic_per_seed():
    d1, _ = run_product(2, [1.0, 1.0], 0.01, 3)
    d2, _ = run_product(2, [1.0, 1.0], 0.01, 3)
    a = d1.arrays()[0]
    b = d2.arrays()[0]
    np.testing.assert_array_equal(a, b)


def test_dart_kernel_follows_pick_points_formula():
    rg = RadiusGenerator(3, [(0.02, 1.0, 0)], volume=1.0)
    dom = Domain([0.0] * 3, [1.0, 1.0, 1.0], 0.02)
    algo = Algo(dom, rg, 6000)
    algo.begin()
    vox, ln, lvl = algo.voxels()
    pos, key, vidx = algo.draw_darts(11, 5, 4096)
    for i in range(0, 4096, 97):
        w = []
        for c in range(3):
            w += list(O.philox4x32_10([i, 5, 0, c], [11, 0]))
        r64 = (int(w[0]) << 32) | int(w[1])
        v = (r64 * len(vox)) >> 64
        assert v == vidx[i]
        for d in range(3):
            bits = ((int(w[2 + 2 * d]) << 32) | int(w[3 + 2 * d])) >> 11
            u = bits * 2.0 ** -53
            orig = 0.0 + float(vox[v, d]) * ln[d]
            assert pos[i, d] == orig + ln[d] * u
        assert key[i] == (int(w[8]) << 32) | i


def _fresh(dim=2, L=(1.0, 1.0), r=0.0625):
    rg = RadiusGenerator(dim, [(r, 10**9, 0)])
    dom = Domain([0.0] * dim, list(L), r)
    algo = Algo(dom, rg, 6000)
    algo.begin()
    return dom, algo


def test_replay_edge_cases():
    """Dyadic coordinates, so that every distance below is exact in FP64."""
    dom, algo = _fresh()
    r = 0.0625
    k = lambda *v: np.array(v, np.uint64) << np.uint64(32)
    # empty round
    acc, n = algo.replay_round(np.zeros((0, 2)), np.zeros(0, np.uint64), np.zeros(0))
    assert n == 0 and len(acc) == 0
    # exact contact is not an overlap (dist^2 == (r1+r2)^2): both accepted
    acc, n = algo.replay_round(np.array([[0.25, 0.5], [0.375, 0.5]]), k(1, 2), np.full(2, r))
    assert list(acc) == [True, True] and n == 2
    # one ulp closer than contact: overlap, the larger priority is rejected
    acc, n = algo.replay_round(np.array([[0.25, 0.75], [np.nextafter(0.375, 0.0), 0.75]]), k(1, 2), np.full(2, r))
    assert list(acc) == [True, False]
    # equal priorities: the candidate index breaks the tie (the reference would accept both, overlapping)
    acc, n = algo.replay_round(np.array([[0.75, 0.25], [0.8125, 0.25]]), k(5, 5), np.full(2, r))
    assert list(acc) == [True, False]
    acc, n = algo.replay_round(np.array([[0.8125, 0.0625], [0.75, 0.0625]]), k(5, 5), np.full(2, r))
    assert list(acc) == [True, False]
    # a chain a < b < c with a-b and b-c overlapping: a and c accepted, b rejected
    acc, n = algo.replay_round(np.array([[0.5, 0.96875], [0.59375, 0.96875], [0.6875, 0.96875]]), k(1, 2, 3),
                               np.full(3, r))
    assert list(acc) == [True, False, True]
    assert dom.check() == (0, 0)


def _pair(form, dim, L, r):
    """A fresh oracle and GPU sampler on the same empty periodic box (one radius, no class count)."""
    ora = O.Oracle(dim, [0.0] * dim, list(L), [(r, 10**9, 0)], counts=True)
    ora.begin(0)
    rg = RadiusGenerator(dim, [(r, 10**9, 0)])
    dom = Domain([0.0] * dim, list(L), r)
    algo = Algo(dom, rg, 6000)
    algo.set_form(form)
    algo.begin()
    return ora, dom, algo


@pytest.mark.parametrize("form", [0, 1], ids=["fp64", "fp32guard"])
def test_reference_cap_follows_the_passes(form):
    """A capped round under the default rule (RSAGPU_CAP_REFERENCE).  B collides with A through the
    periodic boundary only, so in the first pass B is Conflict, and so are E1..E3, which collide with B alone.
    The greedy set is {A, E1, E2, E3}; the reference's first pass validates only A, and the second pass (B
    now hits A and leaves) holds E1..E3.  With a count of 2 the second pass is cut by the pivot: {A, E1, E2},
    where a pivot over the greedy set would keep {A, E1}.  Every pass compares with the round's whole count
    (it is passed by value), so with a bystander D and a count of 3 the round keeps 5 spheres."""
    r = 0.05
    pos = np.array([[0.02, 0.5], [0.97, 0.5], [0.88, 0.5], [0.97, 0.59], [0.97, 0.41]])
    key = np.array([1, 2, 5, 6, 7], np.uint64)
    cases = [(pos, key, 1, [1, 0, 0, 0, 0]), (pos, key, 2, [1, 0, 1, 1, 0]), (pos, key, 3, [1, 0, 1, 1, 1]),
             (pos, key, 10, [1, 0, 1, 1, 1])]
    pos_d = np.vstack([pos, [[0.5, 0.5]]])
    key_d = np.array([1, 2, 5, 6, 7, 3], np.uint64)
    cases += [(pos_d, key_d, 2, [1, 0, 0, 0, 0, 1]), (pos_d, key_d, 3, [1, 0, 1, 1, 1, 1])]
    for p, k, mx, want in cases:
        ora, dom, algo = _pair(form, 2, (1.0, 1.0), r)
        n = len(k)
        acc_o, n_o = ora.apply_round(p, k, np.full(n, r), np.zeros(n, np.int32), mx, 1)
        acc_g, n_g = algo.replay_round(p, k << np.uint64(32), np.full(n, r), max_new=mx, may_outreach=True)
        assert list(acc_o.astype(int)) == want, (mx, acc_o)
        assert list(acc_g.astype(int)) == want, (mx, acc_g)
        assert n_o == n_g == sum(want)
        assert dom.check() == (0, 0)


@pytest.mark.parametrize("form", [0, 1], ids=["fp64", "fp32guard"])
def test_reference_cap_matches_oracle_on_dense_periodic_batches(form):
    """Capped rounds of random candidates in small periodic boxes (many collisions through the boundary,
    Conflict chains, several passes), counts from 5 % to 99 % of the greedy set: the GPU keeps exactly the
    oracle's candidates."""
    rng = np.random.default_rng(21)
    for dim, L, r, n in ((2, (0.3, 0.3), 0.01, 4000), (2, (0.6, 0.5), 0.01, 2500),
                         (3, (0.25, 0.25, 0.25), 0.02, 5000), (4, (0.5, 0.5, 0.5, 0.5), 0.07, 3000)):
        for frac in (0.05, 0.4, 0.8, 0.99):
            pos = rng.random((n, dim)) * np.array(L)
            key = rng.integers(0, 2**24, n).astype(np.uint64)
            rad = np.full(n, r)
            ph = np.zeros(n, np.int32)
            ora, dom, algo = _pair(form, dim, L, r)
            _, greedy = ora.apply_round(pos, key, rad, ph)  # no cap
            mx = max(1, int(frac * greedy))
            ora, dom, algo = _pair(form, dim, L, r)
            acc_o, n_o = ora.apply_round(pos, key, rad, ph, mx, 1)
            acc_g, n_g = algo.replay_round(pos, key << np.uint64(32), rad, max_new=mx, may_outreach=True)
            assert n_o == n_g, (dim, frac, n_o, n_g)
            assert np.array_equal(acc_o, acc_g), (dim, frac, int(np.sum(acc_o != acc_g)))
            assert dom.check() == (0, 0)


def test_replay_periodic_wrap():
    dom, algo = _fresh()
    r = 0.0625
    acc, _ = algo.replay_round(np.array([[0.03125, 0.0625]]), np.array([1], np.uint64), np.full(1, r))
    assert list(acc) == [True]
    # images x + L: across x = 1, across the corner, and exact contact through the boundary
    pos = np.array([[0.9375, 0.0625], [0.96875, 0.96875], [0.90625, 0.5]])
    acc, _ = algo.replay_round(pos, np.array([1, 2, 3], np.uint64), np.full(3, r))
    assert list(acc) == [False, False, True]
    acc, _ = algo.replay_round(np.array([[0.90625, 0.0625]]), np.array([1], np.uint64), np.full(1, r))
    assert list(acc) == [True]  # 0.90625 + 0.125 = 1.03125 = 0.03125 + 1: exact contact
    assert dom.check() == (0, 0)


def test_replay_matches_oracle_on_random_dense_batches():
    """Large random batches with heavy in-batch conflicts and repeated priorities."""
    rng = np.random.default_rng(5)
    for dim, L, r in ((2, [1.0, 1.0], 0.01), (3, [1.0, 0.8, 0.6], 0.03)):
        ora = O.Oracle(dim, [0.0] * dim, L, [(r, 10**9, 0)], counts=True)
        rg = RadiusGenerator(dim, [(r, 10**9, 0)])
        dom = Domain([0.0] * dim, L, r)
        algo = Algo(dom, rg, 6000)
        ora.begin(0)
        algo.begin()
        for rnd in range(4):
            n = 20000
            pos = rng.random((n, dim)) * np.array(L)
            key = rng.integers(0, 2**14, n).astype(np.uint64)  # many ties
            rad = np.full(n, r)
            acc_o, n_o = ora.apply_round(pos, key, rad, np.zeros(n, np.int32))
            acc_g, n_g = algo.replay_round(pos, key << np.uint64(32), rad)
            assert n_o == n_g and np.array_equal(acc_o, acc_g)
        algo.refine()
        ora.refine()
        np.testing.assert_array_equal(sort_voxels(ora.voxels()[0]), sort_voxels(algo.voxels()[0]))
