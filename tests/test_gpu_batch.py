"""The batched form on the GPU: every instance of a batch places exactly the spheres of its own
single-instance run (same count, same centres through an order-free checksum), in both forms, whatever
the wave split and the block shapes."""
import numpy as np
import pytest

from oracle import oracle as O
from rsa_mpi_gb300 import _lib
from rsa_mpi_gb300.sampler import Algo, Domain, RadiusGenerator, batch_run, sphere_checksum

pytestmark = pytest.mark.gpu


def single(dim, sup, r, seed, form):
    rg = RadiusGenerator(dim, [(r, 1.0, 0)], volume=float(np.prod(sup)))
    dom = Domain([0.0] * dim, list(sup), r)
    algo = Algo(dom, rg, 6000)
    algo.set_form(form)
    algo.proceed(seed)
    assert algo.stats()["maximal"] == 1
    pos, rad, _ = dom.arrays()
    return pos, rad


def instances(n_2d=10, n_3d=8, seed=5):
    """Mixed 2D and 3D boxes with log-uniform sides (the batch workload's shape, small sizes)."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n_2d):
        s = float(np.exp(rng.uniform(np.log(0.12), np.log(1.2))))
        out.append((2, [s, s * float(rng.uniform(0.8, 1.25))], 0.02, (1000 + i) << 8 | 3))
    for i in range(n_3d):
        s = float(np.exp(rng.uniform(np.log(0.15), np.log(0.5))))
        out.append((3, [s, s, s * float(rng.uniform(0.8, 1.25))], 0.02, (2000 + i) << 8 | 5))
    return out


@pytest.mark.parametrize("form", [_lib.RSAGPU_FORM_FP32_GUARD, _lib.RSAGPU_FORM_FP64])
def test_batch_instances_equal_their_single_runs(form):
    inst = instances()
    res = batch_run(inst, form=form)
    assert res["stats"]["waves"] >= 2  # one per dimension at least
    for i, (dim, sup, r, seed) in enumerate(inst):
        pos, rad = single(dim, sup, r, seed, form)
        assert int(res["counts"][i]) == len(rad), (i, dim, sup)
        assert int(res["checksums"][i]) == sphere_checksum(pos), (i, dim, sup)
        assert O.count_overlaps(dim, [0.0] * dim, sup, pos, rad) == 0
    assert np.all(res["seconds"] > 0) and np.all(res["seconds"] <= res["stats"]["seconds"] + 1e-9)


def test_batch_results_do_not_depend_on_waves_or_block_shapes():
    inst = instances(6, 6, seed=9)
    a = batch_run(inst, autotune=True)
    b = batch_run(inst, max_bytes=1, autotune=False)  # a budget below any instance: one wave each
    assert a["stats"]["waves"] == 2 and b["stats"]["waves"] == len(inst)
    np.testing.assert_array_equal(a["counts"], b["counts"])
    np.testing.assert_array_equal(a["checksums"], b["checksums"])
    tuned = a["stats"]["block"]
    assert set(tuned) == {2, 3}
    assert all(v in (128, 256, 512) for row in tuned.values() for v in row)


def test_batch_packing_fraction_and_seed_independence():
    # one box, different keys: different packings, each near the saturation fraction of the 2D case
    inst = [(2, [1.0, 1.0], 0.01, k) for k in (1, 2, 3, 4)]
    res = batch_run(inst)
    phi = res["counts"].astype(float) * O.volume_sphere(2, 0.01)
    assert len(set(res["checksums"].tolist())) == 4
    assert np.all(np.abs(phi - 0.547) < 0.01), phi


def test_batch_rejects_bad_instances():
    with pytest.raises(_lib.RsaGpuError):
        batch_run([(2, [0.01, 1.0], 0.02, 1)])  # side below twice the radius
    with pytest.raises(_lib.RsaGpuError):
        batch_run([(9, [1.0] * 7, 0.02, 1)])
    assert batch_run([])["counts"].size == 0
