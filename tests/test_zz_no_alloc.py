"""rsagpu_resolve_batch_noalloc, the conflict-resolution entry point that allocates nothing.

It serves callers that cannot call cudaMalloc (code inside another framework's memory pool, fixed-memory
real-time loops, libraries that must not touch the device heap): they pass device buffers, and the
entry point keeps its temporaries in a static device array of the library.  Its output must equal the
allocating path's (rsagpu_algo_replay_round on an empty domain) decision for decision, on two calls in a
row (the second call runs on the array the first one left behind).  This file is collected last.
"""
import ctypes as C

import numpy as np
import pytest

from rsa_mpi_gb300 import _lib
from rsa_mpi_gb300.sampler import Algo, Domain, RadiusGenerator

pytestmark = pytest.mark.gpu


def _batch(rng, n, dim, L, r):
    pos = rng.random((n, dim)) * np.asarray(L)
    key = (rng.integers(0, 2**20, n).astype(np.uint64) << np.uint64(32))  # repeated priorities too
    rad = np.full(n, r)
    return pos, key, rad


def _allocating_path(pos, key, rad, dim, L, r):
    rg = RadiusGenerator(dim, [(r, 10**12, 0)])
    dom = Domain([0.0] * dim, L, r)
    algo = Algo(dom, rg, 6000)
    algo.begin()
    acc, _ = algo.replay_round(pos, key, rad)
    algo.close()
    dom.close()
    return acc


def _noalloc(pos, key, rad, dim, L, r):
    rc, acc = _noalloc_call(pos, key, rad, dim, L, r)
    _lib.check(rc)
    return acc


def _noalloc_call(pos, key, rad, dim, L, r):
    """(status, decisions) of one call; the decisions buffer starts at 7 in every byte."""
    import torch
    dev = torch.device("cuda:0")
    d_pos = torch.from_numpy(pos).to(dev)
    d_key = torch.from_numpy(key.view(np.int64)).to(dev)
    d_rad = torch.from_numpy(rad).to(dev)
    d_acc = torch.full((len(key),), 7, dtype=torch.uint8, device=dev)
    torch.cuda.synchronize()
    inf = np.zeros(dim)
    sup = np.asarray(L, dtype=np.float64)
    rc = _lib.lib().rsagpu_resolve_batch_noalloc(dim, _lib.ptr(inf, _lib._d), _lib.ptr(sup, _lib._d), r,
                                                 C.c_void_p(d_pos.data_ptr()), C.c_void_p(d_key.data_ptr()),
                                                 C.c_void_p(d_rad.data_ptr()), len(key),
                                                 C.c_void_p(d_acc.data_ptr()), None)
    return rc, d_acc.cpu().numpy()


@pytest.mark.parametrize("dim,L,r", [(2, [1.0, 1.0], 0.004), (3, [1.0, 0.7, 0.5], 0.02)])
def test_noalloc_matches_allocating_path_on_two_calls(dim, L, r):
    rng = np.random.default_rng(2024 + dim)
    for call in range(2):
        n = 200000 if call == 0 else 90000  # the second call is smaller: stale scratch must not leak in
        pos, key, rad = _batch(rng, n, dim, L, r)
        expect = _allocating_path(pos, key, rad, dim, L, r)
        got = _noalloc(pos, key, rad, dim, L, r).astype(bool)
        assert got.sum() > 0
        np.testing.assert_array_equal(got, expect)


def test_noalloc_refuses_radii_above_r_max_and_centres_outside_the_box():
    """The cells are sized from r_max and the box: a larger radius or an outside centre would miss colliders.
    The inputs are in device memory, so the kernel checks them and the call returns RSAGPU_ERR_ARG without
    writing a decision; the next valid call is unaffected."""
    rng = np.random.default_rng(77)
    dim, L, r = 2, [1.0, 1.0], 0.01
    pos, key, rad = _batch(rng, 5000, dim, L, r)
    big = rad.copy()
    big[1234] = np.nextafter(r, 1.0)
    rc, acc = _noalloc_call(pos, key, big, dim, L, r)
    assert rc == _lib.RSAGPU_ERR_ARG and np.all(acc == 7)
    assert "r_max" in _lib.lib().rsagpu_last_error().decode()
    out = pos.copy()
    out[4321, 1] = 1.25
    rc, acc = _noalloc_call(out, key, rad, dim, L, r)
    assert rc == _lib.RSAGPU_ERR_ARG and np.all(acc == 7)
    assert "outside" in _lib.lib().rsagpu_last_error().decode()
    got = _noalloc(pos, key, rad, dim, L, r).astype(bool)
    np.testing.assert_array_equal(got, _allocating_path(pos, key, rad, dim, L, r))


def test_noalloc_refuses_batches_above_its_limit():
    import torch
    n = _lib.lib  # noqa: F841
    limit = 1 << 18
    inf = np.zeros(2)
    sup = np.ones(2)
    dummy = torch.zeros(1, dtype=torch.float64, device="cuda:0")
    rc = _lib.lib().rsagpu_resolve_batch_noalloc(2, _lib.ptr(inf, _lib._d), _lib.ptr(sup, _lib._d), 0.01,
                                                 C.c_void_p(dummy.data_ptr()), C.c_void_p(dummy.data_ptr()),
                                                 C.c_void_p(dummy.data_ptr()), limit + 1,
                                                 C.c_void_p(dummy.data_ptr()), None)
    assert rc == -7
    assert "RSAGPU_NOALLOC_MAX_CANDIDATES" in _lib.lib().rsagpu_last_error().decode()
