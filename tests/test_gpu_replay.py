"""Decision parity of the CUDA path with the FP64 oracle, fed the reference's own candidate stream.

The oracle (oracle/rsa_oracle.c) draws each round exactly as the reference does (mt19937 stream,
Poisson shot count, pick_points, priorities); the GPU decides the same candidates through the C ABI
(rsagpu_algo_replay_round) and refines its own voxel list (rsagpu_algo_end_round).  Every accept/reject
decision and every voxel set after a refinement must be identical, and at the end the GPU's sphere set
must equal the reference's own output (tests/golden/, made by the reference compiled here).
"""
import numpy as np
import pytest

from oracle import oracle as O
from gpu_helpers import GOLDEN, INDEX, drive, lockstep, make_pair, sort_spheres
from rsa_mpi_gb300.sampler import RadiusGenerator

pytestmark = pytest.mark.gpu

MONO = ["c1_2d_r0.005_s0", "t2d_r0.05_s0", "t3d_r0.05_s0", "k3d_r0.02_s1", "t3d_box3.5_r0.4_s0", "n2d_rect_s7"]
# continuous radius law (RandomRadiusGenerator, uniform transform): per-dart radii from the reference's stream
UNIFORM = ["u3d_r0.05-0.055_s0", "u2d_r0.02-0.025_s7", "u2d_r0.01-0.0105_s3"]


@pytest.mark.parametrize("form", [0, 1], ids=["fp64", "fp32guard"])
@pytest.mark.parametrize("name", MONO + UNIFORM)
def test_replay_reproduces_reference_output(name, form):
    case = INDEX[name]
    g = np.load(f"{GOLDEN}/{name}.npz")
    ora, algo, dom, rounds = lockstep(case, case["seed"], form=form)
    assert rounds == len(g["shots"])
    pos, rad, ph = sort_spheres(*dom.arrays())
    np.testing.assert_array_equal(pos, g["centers"])
    np.testing.assert_array_equal(rad, g["radii"])
    np.testing.assert_array_equal(ph, g["phases"])
    assert dom.check() == (0, 0)
    # certified maximal: the voxel list is empty at exit
    assert len(algo.voxels()[0]) == 0


@pytest.mark.parametrize("form", [0, 1], ids=["fp64", "fp32guard"])
@pytest.mark.parametrize("name", ["p2d_poly_s3", "t3d_radius_s0", "p3d_poly_small_s2"])
def test_replay_polydisperse_exact_cap(name, form):
    """Class counts reached inside a round: both sides keep exactly the remaining count."""
    case = INDEX[name]
    ora, algo, dom, rounds = lockstep(case, case["seed"], cap_exact=True, form=form)
    po, ro, fo = sort_spheres(*ora.spheres())
    pg, rg, fg = sort_spheres(*dom.arrays())
    np.testing.assert_array_equal(po, pg)
    np.testing.assert_array_equal(ro, rg)
    np.testing.assert_array_equal(fo, fg)
    vol = 1.0 if case["volume_mode"] == 1 else float(np.prod(case["L"]))
    counts = [O.count_from_fraction(case["dim"], r, phi, vol) for r, phi, _ in case["classes"]]
    np.testing.assert_array_equal(np.bincount(fg, minlength=len(counts)), counts)


@pytest.mark.parametrize("form", [0, 1], ids=["fp64", "fp32guard"])
@pytest.mark.parametrize("name", ["p2d_poly_s3", "t3d_radius_s0"])
def test_replay_polydisperse_reference_cap(name, form):
    """The count-cap rule every product run uses by default (RSAGPU_CAP_REFERENCE): a capped round goes
    through the reference's passes on the device, each pass's Undecided set compared with the class count and
    cut by the pivot priority.  Every decision and voxel set equals the oracle's, and the final sphere set and
    round count equal the reference's own output bit for bit."""
    case = INDEX[name]
    g = np.load(f"{GOLDEN}/{name}.npz")
    ora, algo, dom, rounds = lockstep(case, case["seed"], form=form)
    assert rounds == len(g["shots"])
    pos, rad, ph = sort_spheres(*dom.arrays())
    np.testing.assert_array_equal(pos, g["centers"])
    np.testing.assert_array_equal(rad, g["radii"])
    np.testing.assert_array_equal(ph, g["phases"])
    assert dom.check() == (0, 0)


@pytest.mark.parametrize("form", [0, 1], ids=["fp64", "fp32guard"])
@pytest.mark.parametrize("name,seed", [("p2d_poly_s3", s) for s in (None, 11, 12, 13, 14, 17)] +
                         [("p3d_poly_small_s2", s) for s in (None, 12, 15)])
def test_replay_reference_cap_against_oracle(name, seed, form):
    """The default count-cap rule on more class transitions, against the oracle round by round (each of these
    seeds has capped rounds where the rule keeps another set than an exact cut would).  The 3D three-class
    case at its golden seed (2) meets a capped round in which a candidate has both a collider through the
    periodic boundary and an ordinary one; the reference's outcome there follows its cell-scan order, so that
    case is checked against the oracle (Conflict wins), with the reference's sphere count."""
    case = INDEX[name]
    ora, algo, dom, rounds = lockstep(case, case["seed"] if seed is None else seed, form=form)
    po, ro, fo = sort_spheres(*ora.spheres())
    pg, rg, fg = sort_spheres(*dom.arrays())
    np.testing.assert_array_equal(po, pg)
    np.testing.assert_array_equal(ro, rg)
    np.testing.assert_array_equal(fo, fg)
    assert dom.check() == (0, 0)
    if seed is None:
        assert len(rg) == case["n_spheres"]


@pytest.mark.parametrize("form", [0, 1], ids=["fp64", "fp32guard"])
@pytest.mark.parametrize("seed", [11, 13])
@pytest.mark.parametrize("name", ["p2d_poly_s3", "p3d_poly_small_s2"])
def test_replay_polydisperse_other_seeds(name, seed, form):
    """More class transitions: the GPU's grid is rebuilt for each smaller class (cells sized for the radii
    placed so far) and the candidate searches reach the round's class radius; every decision and voxel set
    still matches the oracle round by round."""
    case = INDEX[name]
    ora, algo, dom, rounds = lockstep(case, seed, cap_exact=True, form=form)
    po, ro, fo = sort_spheres(*ora.spheres())
    pg, rg, fg = sort_spheres(*dom.arrays())
    np.testing.assert_array_equal(po, pg)
    np.testing.assert_array_equal(ro, rg)
    np.testing.assert_array_equal(fo, fg)
    assert dom.check() == (0, 0)


@pytest.mark.parametrize("form", [0, 1], ids=["fp64", "fp32guard"])
@pytest.mark.parametrize("dim,L,lo,hi,seed", [(2, [1.0, 1.0], 0.01, 0.02, 3), (3, [1.0, 0.8, 0.6], 0.04, 0.06, 5)])
def test_replay_tabulated_radius_law(dim, L, lo, hi, seed, form):
    """An arbitrary transform of the reference's RandomRadiusGenerator, tabulated (log-uniform radii between lo
    and hi at 4,097 knots): the oracle draws each round's radii from the reference's stream through the table,
    and the GPU decides the same candidates and refines the same voxels, to maximality."""
    knots = lo * (hi / lo) ** np.linspace(0.0, 1.0, 4097)
    case = {"dim": dim, "nbshots": 6000, "L": L, "table": (knots, 10**16, 2)}
    ora, algo, dom, rounds = lockstep(case, seed, form=form)
    po, ro, fo = sort_spheres(*ora.spheres())
    pg, rg, fg = sort_spheres(*dom.arrays())
    np.testing.assert_array_equal(po, pg)
    np.testing.assert_array_equal(ro, rg)
    assert np.all(fg == 2) and ro.min() >= lo and ro.max() <= hi
    assert len(algo.voxels()[0]) == 0 and dom.check() == (0, 0)


@pytest.mark.parametrize("form", [0, 1], ids=["fp64", "fp32guard"])
@pytest.mark.parametrize("dim,r,seed", [(4, 0.12, 3), (4, 0.12, 4), (5, 0.2, 3)])
def test_replay_higher_dimensions_against_oracle(dim, r, seed, form):
    """D = 4 and 5, decision by decision and voxel set by voxel set against the oracle, to certified
    maximality.  The reference's own corner table for D >= 4 (auxiliary/Path.ixx:105-114) writes out of bounds
    and never sets dimension 0, so its subdivision keeps half of each voxel's children, each twice; the oracle
    and the GPU list all 2^D children (bit d of the child index), and parity in D >= 4 is against the oracle."""
    case = {"dim": dim, "nbshots": 6000, "volume_mode": 0, "L": [1.0] * dim, "classes": [[r, 1.0, 0]]}
    ora, algo, dom, rounds = lockstep(case, seed, form=form)
    po, ro, fo = sort_spheres(*ora.spheres())
    pg, rg, fg = sort_spheres(*dom.arrays())
    np.testing.assert_array_equal(po, pg)
    np.testing.assert_array_equal(ro, rg)
    vg, _, level = algo.voxels()
    assert len(vg) == 0 and len(ora.voxels()[0]) == 0
    assert level == ora.voxel_level > 0
    assert dom.check() == (0, 0)


@pytest.mark.parametrize("form", [0, 1], ids=["fp64", "fp32guard"])
@pytest.mark.parametrize("name", ["r2d_r0.02x0.7_s1", "r3d_r0.05x0.8_s2"])
def test_replay_reiteration_reproduces_reference_output(name, form):
    """reset_radius_generator with a smaller radius on the same domain, then proceed again: the grid is
    rebuilt for the new radius, the voxel lattice keeps the algorithm's largest r_max, and after every stage
    the sphere sets agree; the final set equals the reference's own output."""
    case = INDEX[name]
    g = np.load(f"{GOLDEN}/{name}.npz")
    mult, steps = case["reiterate"]
    rad = case["classes"][0][0]
    ora, algo, dom = make_pair(case, form=form)
    D = case["dim"]
    vol = float(np.prod(case["L"]))
    for stage in range(steps + 1):
        if stage:
            rad *= mult
            ora.reset([(rad, 1.0, 0)], volume=vol)
            algo.reset_radius_generator(RadiusGenerator(D, [(rad, 1.0, 0)], volume=vol))
        drive(ora, algo, case["seed"])
        po, ro, fo = sort_spheres(*ora.spheres())
        pg, rg, fg = sort_spheres(*dom.arrays())
        np.testing.assert_array_equal(po, pg)
        np.testing.assert_array_equal(ro, rg)
        assert len(algo.voxels()[0]) == 0
    np.testing.assert_array_equal(pg, g["centers"])
    np.testing.assert_array_equal(rg, g["radii"])
    np.testing.assert_array_equal(fg, g["phases"])
    assert dom.check() == (0, 0)


@pytest.mark.parametrize("form", [0, 1], ids=["fp64", "fp32guard"])
def test_replay_reiteration_with_radius_classes(form):
    """reset_radius_generator between two generators of two classes each: the GPU's grid is staged for each
    class, and again at the reset for the second generator's first class; every decision and voxel set agrees
    with the oracle, and so do the sphere sets after each proceed."""
    case = {"dim": 2, "nbshots": 2000, "volume_mode": 0, "L": [1.0, 1.0],
            "classes": [[0.02, 0.25, 0], [0.01, 0.1, 1]]}
    ora, algo, dom = make_pair(case, cap_exact=True, form=form)
    second = [(0.008, 0.04, 2), (0.004, 0.02, 3)]
    for stage in range(2):
        if stage:
            ora.reset(second, volume=1.0)
            algo.reset_radius_generator(RadiusGenerator(2, second, volume=1.0))
        drive(ora, algo, 5 + stage)
        po, ro, fo = sort_spheres(*ora.spheres())
        pg, rg, fg = sort_spheres(*dom.arrays())
        np.testing.assert_array_equal(po, pg)
        np.testing.assert_array_equal(ro, rg)
        np.testing.assert_array_equal(fo, fg)
    assert set(np.unique(fg).tolist()) == {0, 1, 2, 3}
    assert dom.check() == (0, 0)


@pytest.mark.parametrize("name", ["t2d_r0.05_s0", "t3d_r0.05_s0"])
def test_replayed_output_files_list_the_reference_cells_in_order(name, tmp_path):
    """The spheres of a replayed run, written with the reference's cell order: the same cell sequence as the
    reference's own files, the same spheres in every cell, and the same bytes wherever the order within a
    cell agrees (one sphere per cell, or the same acceptance order)."""
    import os
    from rsa_mpi_gb300 import writers as W
    case = INDEX[name]
    ora, algo, dom, rounds = lockstep(case, case["seed"])
    inf, sup, rad = [0.0] * case["dim"], case["L"], case["classes"][0][0]
    pos, r, ph = W.reference_order(*dom.arrays(), inf, sup, rad)
    g = np.load(f"{GOLDEN}/writers/{name}/order.npz")
    kg = W.reference_cell_keys(pos, inf, sup, rad)
    np.testing.assert_array_equal(kg, W.reference_cell_keys(g["centers"], inf, sup, rad))
    for k in np.unique(kg):  # the same spheres in every cell
        sel = kg == k
        np.testing.assert_array_equal(sort_spheres(pos[sel], r[sel], ph[sel])[0],
                                      sort_spheres(g["centers"][sel], g["radii"][sel], g["phases"][sel])[0])
    W._step[0] = 0
    W.write_paraview(str(tmp_path / "pv"), pos, r, ph)
    W.write_vtk(str(tmp_path / "spheres.vtk"), pos, r, np.zeros_like(ph))
    ref = open(f"{GOLDEN}/writers/{name}/spheres.vtk").read().splitlines()
    out = open(tmp_path / "spheres.vtk").read().splitlines()
    assert sorted(ref) == sorted(out) and ref[:5] == out[:5]
    same = np.all(pos == g["centers"], axis=1)
    assert same.mean() > 0.5
    assert open(f"{GOLDEN}/writers/{name}/pv/rsa_mpi_0.pvtp").read() == open(tmp_path / "pv" / "rsa_mpi_0.pvtp").read()
    assert os.path.exists(tmp_path / "pv" / "rsa_mpi_0" / "rsa_mpi_0_0.vtp")
