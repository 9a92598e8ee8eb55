"""Shared helpers of the GPU tests: lockstep replay of the oracle's candidate stream."""
import json
import os

import numpy as np

from oracle import oracle as O
from rsa_mpi_gb300 import _lib
from rsa_mpi_gb300.sampler import Algo, Domain, RadiusGenerator

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
INDEX = json.load(open(os.path.join(GOLDEN, "index.json")))


def sort_spheres(pos, rad, ph):
    order = np.lexsort(tuple(pos[:, d] for d in reversed(range(pos.shape[1]))))
    return pos[order], rad[order], ph[order]


def sort_voxels(v):
    if len(v) == 0:
        return v
    return v[np.lexsort(tuple(v[:, d] for d in reversed(range(v.shape[1]))))]


def make_pair(case, cap_exact=False, form=0):
    """(oracle, gpu algo, gpu domain) for a golden case."""
    D = case["dim"]
    if "table" in case:  # continuous radius law, tabulated transform
        knots, count, ph = case["table"]
        ora = O.Oracle.table(D, [0.0] * D, case["L"], knots, count, ph, nbshots=case["nbshots"])
        rg = RadiusGenerator.transform(D, lambda x: float(np.interp(x, np.linspace(0, 1, len(knots)), knots)),
                                       count, ph, knots=len(knots))
        dom = Domain([0.0] * D, case["L"], rg.max_radius)
        algo = Algo(dom, rg, case["nbshots"])
        algo.set_form(form)
        return ora, algo, dom
    if "uniform" in case:  # continuous radius law
        r0, r1, count, ph = case["uniform"]
        ora = O.Oracle.uniform(D, [0.0] * D, case["L"], r0, r1, count, ph, nbshots=case["nbshots"])
        rg = RadiusGenerator.uniform(D, r0, r1, count, ph)
        dom = Domain([0.0] * D, case["L"], rg.max_radius)
        algo = Algo(dom, rg, case["nbshots"])
        algo.set_form(form)
        return ora, algo, dom
    vol = 1.0 if case["volume_mode"] == 1 else float(np.prod(case["L"]))
    classes = [tuple(x) for x in case["classes"]]
    ora = O.Oracle(D, [0.0] * D, case["L"], classes, nbshots=case["nbshots"], volume=vol)
    if cap_exact:
        O.lib().ora_set_cap_exact(ora._h, 1)
    rg = RadiusGenerator(D, classes, volume=vol)
    dom = Domain([0.0] * D, case["L"], rg.max_radius)
    algo = Algo(dom, rg, case["nbshots"])
    algo.set_form(form)
    if cap_exact:
        algo.set_cap_rule(_lib.RSAGPU_CAP_EXACT)
    return ora, algo, dom


def lockstep(case, seed, cap_exact=False, check_voxels=True, max_rounds=100000, form=0):
    """Drives the oracle and the GPU with the reference's own candidate stream; asserts equal decisions
    every round and equal voxel sets after every refinement.  Returns (oracle, algo, dom, rounds)."""
    ora, algo, dom = make_pair(case, cap_exact, form)
    return (ora, algo, dom) + (drive(ora, algo, seed, check_voxels, max_rounds),)


def drive(ora, algo, seed, check_voxels=True, max_rounds=100000):
    """One proceed of both sides in lockstep (see lockstep); returns the number of rounds."""
    ora.begin(seed)
    algo.begin()
    rounds = 0
    for _ in range(max_rounds):
        st, cand, mx, may = ora.gen_round()
        if st != 0:
            break
        n = len(cand["key"])
        if n == 0:
            continue
        keys = cand["key"].astype(np.uint64) << np.uint64(32)
        acc_o, n_o = ora.apply_round(cand["pos"], cand["key"], cand["rad"], cand["phase"], mx, may)
        acc_g, n_g = algo.replay_round(cand["pos"], keys, cand["rad"], cand["phase"], mx, may)
        assert n_o == n_g, f"round {rounds}: oracle accepted {n_o}, GPU {n_g}"
        assert np.array_equal(acc_o, acc_g), f"round {rounds}: {int(np.sum(acc_o != acc_g))} decisions differ"
        done_o, ref_o = ora.end_round(n, n_o)
        done_g, ref_g = algo.end_round(n, n_g)
        assert ref_o == ref_g and done_o == done_g
        if ref_o and check_voxels:
            vo, lo = ora.voxels()
            vg, lg, _ = algo.voxels()
            assert len(vo) == len(vg), f"round {rounds}: {len(vo)} voxels vs {len(vg)}"
            np.testing.assert_array_equal(lo, lg)
            np.testing.assert_array_equal(sort_voxels(vo), sort_voxels(vg))
        rounds += 1
        if done_o:
            break
    return rounds
