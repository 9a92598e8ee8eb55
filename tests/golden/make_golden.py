"""Generates the golden fixtures of tests/golden/ from the REFERENCE itself.

Runs oracle/_ref/ref_rsa (the reference sampler compiled from its own headers
against the single-rank MPI stand-in, see oracle/Makefile) on each case below
and stores, per case, the sphere set sorted lexicographically by centre, the
packing volume and the per-round trace the reference prints (shots, misses,
voxels after the round).  Needs the reference checkout, so it runs in the
development container only; the fixtures it writes are committed.

    python tests/golden/make_golden.py [--reference /path/to/RSA_MPI]
"""
from __future__ import annotations

import argparse
import json
import os
import re
import subprocess
import tempfile
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

# name -> (dim, seed, nbshots, volume_mode, L, classes[(r, phi, phase)])
# volume_mode 0: class counts from the box volume (rsa_algo::uniform_generate);
# volume_mode 1: volume 1 whatever the box (the reference's ::throw_spheres / test_ND_radius).
CASES = {
    # BASELINE config 1: 2D periodic unit square, r = 0.005, seed 0
    "c1_2d_r0.005_s0": (2, 0, 6000, 0, [1.0, 1.0], [(0.005, 1.0, 0)]),
    # reference test test_2D_full_voxel.cpp:9 (test_ND<2,1>(0.05), seed 0)
    "t2d_r0.05_s0": (2, 0, 6000, 0, [1.0, 1.0], [(0.05, 1.0, 0)]),
    # reference test test_3D_full_voxel.cpp:9 (test_ND<3,1>(0.05), seed 0)
    "t3d_r0.05_s0": (3, 0, 6000, 0, [1.0, 1.0, 1.0], [(0.05, 1.0, 0)]),
    # 3D r = 0.02 seed 1 (survey known answer: 11,495 spheres)
    "k3d_r0.02_s1": (3, 1, 6000, 0, [1.0, 1.0, 1.0], [(0.02, 1.0, 0)]),
    # reference test test_3D_radius.cpp:9-10 (test_ND_radius<3,1>, volume 1, seed 0)
    "t3d_radius_s0": (3, 0, 6000, 1, [1.0, 1.0, 1.0], [(0.25, 0.1, 0), (0.125, 0.1, 1)]),
    # polydisperse, nonincreasing radii with target fractions (config-3 shape at 1/10 scale)
    "p3d_poly_s1": (3, 1, 6000, 0, [1.0, 1.0, 1.0], [(0.04, 0.20, 0), (0.02, 0.10, 1), (0.01, 0.05, 2)]),
    # polydisperse at 1/20 scale of the count (fast enough for the default CPU suite)
    "p3d_poly_small_s2": (3, 2, 6000, 0, [1.0, 1.0, 1.0], [(0.08, 0.20, 0), (0.04, 0.10, 1), (0.02, 0.05, 2)]),
    "p2d_poly_s3": (2, 3, 2000, 0, [1.0, 1.0], [(0.02, 0.30, 0), (0.01, 0.15, 1), (0.005, 0.05, 2)]),
    # reference test test_python.cpp:8-31 (box 3.5^3, r = 0.4, seed 0)
    "t3d_box3.5_r0.4_s0": (3, 0, 6000, 0, [3.5, 3.5, 3.5], [(0.4, 1.0, 0)]),
    # non-cubic 2D box, small nbshots (many rounds)
    "n2d_rect_s7": (2, 7, 500, 0, [1.3, 0.7], [(0.02, 1.0, 0)]),
}

# cases whose reference output files (ParaView, legacy VTK, XYZ) are kept under writers/<name>/, with the
# spheres in the reference's own extraction order (Real cells in traversal order) as writers/<name>/order.npz
WRITER_CASES = ["t2d_r0.05_s0", "t3d_r0.05_s0", "t3d_radius_s0"]

# continuous radius law (sac_de_billes::RandomRadiusGenerator, radius = r_min + (r_max - r_min) x):
# name -> (dim, seed, nbshots, L, r_min, r_max, count, phase); count 10^16 runs to maximality
UNIFORM_CASES = {
    # the uniform law of the reference test test_random_radius_generator.cpp:13-29 (3D, r in [0.05, 0.055])
    "u3d_r0.05-0.055_s0": (3, 0, 6000, [1.0, 1.0, 1.0], 0.05, 0.055, 10**16, 0),
    "u2d_r0.02-0.025_s7": (2, 7, 6000, [1.0, 1.0], 0.02, 0.025, 10**16, 0),
    "u2d_r0.01-0.0105_s3": (2, 3, 3000, [1.0, 1.0], 0.01, 0.0105, 10**16, 1),
}


# re-iteration (scripts/main_max_frac.cpp:30-60): a maximal run with r_0, then <steps> runs with the radius
# multiplied by <multiplier>, reset_radius_generator and proceed(seed) on the same domain:
# name -> (dim, seed, nbshots, L, r_0, multiplier, steps)
REITER_CASES = {
    "r2d_r0.02x0.7_s1": (2, 1, 6000, [1.0, 1.0], 0.02, 0.7, 3),
    "r3d_r0.05x0.8_s2": (3, 2, 6000, [1.0, 1.0, 1.0], 0.05, 0.8, 2),
}


def parse_trace(log: str):
    shots = [int(m.group(1)) for m in re.finditer(r"--> Miss rate = .*?Nb shots = (\d+) ; Nb miss", log)]
    miss = [int(m.group(1)) for m in re.finditer(r"--> Miss rate = .*?Nb miss =\s+(\d+)", log)]
    vox = [int(m.group(1)) for m in re.finditer(r"Total nb voxels: (\d+)", log)]
    return np.array(shots, np.int64), np.array(miss, np.int64), np.array(vox, np.int64)


def sort_spheres(c, r, p):
    order = np.lexsort(tuple(c[:, d] for d in reversed(range(c.shape[1]))))
    return c[order], r[order], p[order]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("RSA_REFERENCE", "/root/reference"))
    ap.add_argument("--only", default=None)
    args = ap.parse_args()
    ref = O.build_ref(args.reference)
    if ref is None:
        sys.exit("reference checkout not found")
    index_path = os.path.join(HERE, "index.json")
    index = json.load(open(index_path)) if args.only and os.path.exists(index_path) else {}
    jobs = [(name, spec, None) for name, spec in CASES.items()]
    jobs += [(name, (dim, seed, nbshots, 0, L, []), (r0, r1, count, ph))
             for name, (dim, seed, nbshots, L, r0, r1, count, ph) in UNIFORM_CASES.items()]
    jobs += [(name, (dim, seed, nbshots, 0, L, [(r0, 1.0, 0)]), ("reiter", mult, steps))
             for name, (dim, seed, nbshots, L, r0, mult, steps) in REITER_CASES.items()]
    tmp = tempfile.mkdtemp(prefix="rsa_golden_")
    for name, (dim, seed, nbshots, vmode, L, classes), uniform in jobs:
        if args.only and args.only != name:
            continue
        out = os.path.join(tmp, f"golden_{name}.bin")
        if uniform is None:
            cmd = [ref, "run", str(dim), str(seed), str(nbshots), str(vmode)] + [repr(x) for x in L]
            cmd += [str(len(classes))]
            for r, phi, ph in classes:
                cmd += [repr(r), repr(phi), str(ph)]
        elif uniform[0] == "reiter":
            _, mult, steps = uniform
            cmd = [ref, "reiter", str(dim), str(seed), str(nbshots)] + [repr(x) for x in L]
            cmd += [repr(classes[0][0]), repr(mult), str(steps)]
        else:
            r0, r1, count, ph = uniform
            cmd = [ref, "runu", str(dim), str(seed), str(nbshots)] + [repr(x) for x in L]
            cmd += [repr(r0), repr(r1), str(count), str(ph)]
        cmd += [out]
        env = dict(os.environ, OMP_NUM_THREADS="8")
        env.pop("RSA_REF_OUTPUTS", None)
        wdir = os.path.join(HERE, "writers", name)
        if name in WRITER_CASES:
            os.makedirs(wdir, exist_ok=True)
            env["RSA_REF_OUTPUTS"] = wdir
        log = subprocess.run(cmd, check=True, capture_output=True, text=True, env=env).stdout
        c, r, p = O.read_ref_spheres(out)
        if name in WRITER_CASES:
            np.savez_compressed(os.path.join(wdir, "order.npz"), centers=c, radii=r, phases=p)
        c, r, p = sort_spheres(c, r, p)
        shots, miss, vox = parse_trace(log)
        vol = float(re.search(r"volume_of_spheres (\S+)", log).group(1))
        secs = float(re.search(r"proceed_seconds (\S+)", log).group(1))
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), centers=c, radii=r, phases=p,
                            shots=shots, miss=miss, voxels=vox)
        index[name] = dict(dim=dim, seed=seed, nbshots=nbshots, volume_mode=vmode, L=L,
                           classes=[list(x) for x in classes], n_spheres=int(len(r)),
                           volume_of_spheres=vol, rounds=int(len(shots)), ref_seconds_8threads=secs)
        if uniform is not None and uniform[0] == "reiter":
            index[name]["reiterate"] = [uniform[1], uniform[2]]
        elif uniform is not None:
            index[name]["uniform"] = list(uniform)
        print(name, len(r), vol, len(shots), f"{secs:.3f}s")
    with open(index_path, "w") as f:
        json.dump(index, f, indent=1)


if __name__ == "__main__":
    main()
