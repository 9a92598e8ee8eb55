"""Benchmark: spheres/s to certified maximality on one GB300 (and N replicas for N GPUs).

Workload (one step): the 3D periodic unit cube, monodisperse r = 0.002, seed 1, sampled to certified
maximality (no uncovered voxel left) by the FP32 guard-band GPU form (--form 1, the default; --form 0 is the
plain FP64 form, whose output is the same sphere for sphere) -- about 11.5 M spheres.  Inputs are
the configuration only; the working set (sphere grid 434^3 cells, voxel lists of 10^8+ entries) is far
larger than L2, so no flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference] [--workload NAME]

value  = spheres placed / device time of proceed() (CUDA events on the sampler's stream), summed over
         ranks, divided by the max over ranks.
e2e    = the same metric through the C ABI as a user calls it: create domain + algo, proceed, copy the
         spheres (centres, radii, phases) to host buffers, destroy; timed on the host clock.
roofline: the refinement mask kernel (the dominant kernel), algorithmic bytes / its CUDA-event time,
         against the measured HBM copy bandwidth of this GPU.
cpu_baseline: the oracle's C restatement of the reference (single thread) on a bounded sample of the
         same workload (same radius, periodic box of side 0.2 = 1/125 of the volume).
--impl reference: the CPU path of the reference, restated by the oracle (the reference itself cannot
         be compiled on the GPU host, which has no copy of its sources): one instance per host core on
         the bounded sample, run concurrently; the line reports their aggregate spheres/s.  Against the
         reference compiled unmodified (x86, 8 cores, same sample) the restatement ran at 1.17x the
         reference's speed on one thread and 0.81x for 8 concurrent instances (REFERENCE_CALIBRATION).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "spheres/s to certified maximality"
WORKLOADS = {
    # name: (dim, L, r, seed, description)
    "config2": (3, [1.0, 1.0, 1.0], 0.002, 1, "3D periodic unit cube, r=0.002, seed 1, to certified maximality"),
    "3d_r0.004": (3, [1.0, 1.0, 1.0], 0.004, 1, "3D periodic unit cube, r=0.004, seed 1, to certified maximality"),
    "config1": (2, [1.0, 1.0], 0.005, 0, "2D periodic unit square, r=0.005, seed 0, to certified maximality"),
}
CPU_SAMPLE = (3, [0.2, 0.2, 0.2], 0.002, 1)
# the oracle's restatement against the reference itself on CPU_SAMPLE (Intel Xeon @ 2.70 GHz, 8 cores, median
# of 3): reference 7.58 s on 1 OpenMP thread, restatement 6.49 s; 8 concurrent 1-thread instances 8.08 s
# (reference) against 9.97 s (restatement)
REFERENCE_CALIBRATION = {"cpu": "Intel Xeon @ 2.70 GHz, 8 cores", "port_vs_reference_1_thread": 1.17,
                         "port_vs_reference_8_instances": 0.81}


def env_rank():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            j = json.load(f)
        return float(j["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        fd, self.path = tempfile.mkstemp(prefix="rsa_bench_clocks_", suffix=".csv")
        os.close(fd)

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait()
            self.f.close()

    def summary(self):
        try:
            rows = [l.strip().split(",") for l in open(self.path) if l.strip()]
        except Exception:
            return None
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
                for n, v in zip(names, r[5:9]):
                    if v.strip() == "Active":
                        reasons.add(n)
            except (ValueError, IndexError):
                continue
        try:
            os.unlink(self.path)
        except OSError:
            pass
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


FORM_NAMES = {0: "plain FP64", 1: "FP32 screen + FP64 guard-band retest"}
# the mask pass: one kernel per launch (FP32 form, 3D: the cooperative kernel at level 0, the warp queue below);
# FORM_TRAFFIC names its entry in profiles/refine_mask_traffic.json
FORM_KERNEL = {0: "k_refine_mask", 1: "k_refine_mask32c (level 0) + k_refine_mask32q (levels >= 1)"}
FORM_TRAFFIC = {0: "k_refine_mask", 1: "mask_pass_fp32"}


def aggregate(times, counts, dist=None, device="cpu"):
    """Whole-job figures of N replicas: the max over ranks of each time, the sum of each count."""
    import torch
    t = torch.tensor(times, dtype=torch.float64, device=device)
    c = torch.tensor(counts, dtype=torch.float64, device=device)
    if dist is not None:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dist.all_reduce(c, op=dist.ReduceOp.SUM)
    return t.tolist(), c.tolist()


def run_gpu_step(dim, L, r, seed, form=1, checksum=False):
    """One run to maximality: (spheres, stats, mask-pass ms / bytes / voxels per launch[, centre checksum])."""
    from rsa_mpi_gb300.sampler import Algo, Domain, RadiusGenerator, sphere_checksum
    rg = RadiusGenerator(dim, [(r, 1.0, 0)], volume=float(math.prod(L)))
    dom = Domain([0.0] * dim, L, r)
    algo = Algo(dom, rg, 6000)
    algo.set_form(form)
    algo.proceed(seed)
    st = algo.stats()
    ms, by, vx = algo.kernel_profile()
    n = dom.count()
    out = (n, st, ms, by, vx)
    if checksum:
        out += (sphere_checksum(dom.arrays()[0]),)
    algo.close()
    dom.close()
    return out


def pinned_outputs(dim, cap):
    """Pinned host buffers for the spheres (centres, radii, phases), allocated once outside the timed region."""
    import torch
    return (torch.empty((cap, dim), dtype=torch.float64, pin_memory=True).numpy(),
            torch.empty(cap, dtype=torch.float64, pin_memory=True).numpy(),
            torch.empty(cap, dtype=torch.int32, pin_memory=True).numpy())


def run_e2e_step(dim, L, r, seed, form=1, out=None):
    """The user's call through the C ABI with host buffers: returns (spheres, seconds, d2h bytes).  out: pinned
    buffers (pinned_outputs) the spheres are read into, when they are large enough."""
    import ctypes as C
    import numpy as np
    from rsa_mpi_gb300 import _lib
    Lb = _lib.lib()
    t0 = time.perf_counter()
    inf = np.zeros(dim)
    sup = np.asarray(L, dtype=np.float64)
    dom = C.c_void_p()
    _lib.check(Lb.rsagpu_domain_create(dim, _lib.ptr(inf, _lib._d), _lib.ptr(sup, _lib._d), r, C.byref(dom)))
    rr = np.array([r])
    phi = np.array([1.0])
    ph = np.zeros(1, np.int32)
    rg = C.c_void_p()
    _lib.check(Lb.rsagpu_radgen_create_fractions(dim, _lib.ptr(rr, _lib._d), _lib.ptr(phi, _lib._d), _lib.ptr(ph, _lib._i32),
                                                 1, float(np.prod(sup)), 0.0, C.byref(rg)))
    algo = C.c_void_p()
    _lib.check(Lb.rsagpu_algo_create(dom, rg, 6000, C.byref(algo)))
    _lib.check(Lb.rsagpu_algo_set_form(algo, form, 0))
    _lib.check(Lb.rsagpu_algo_proceed(algo, seed))
    n = C.c_uint64()
    _lib.check(Lb.rsagpu_domain_extract(dom, None, None, None, 0, C.byref(n)))
    k = n.value
    if out is not None and len(out[1]) >= k:
        pos, rad, phs = out[0][:k], out[1][:k], out[2][:k]
    else:
        pos = np.empty((k, dim))
        rad = np.empty(k)
        phs = np.empty(k, np.int32)
    _lib.check(Lb.rsagpu_domain_extract(dom, _lib.ptr(pos, _lib._d), _lib.ptr(rad, _lib._d), _lib.ptr(phs, _lib._i32), k,
                                        C.byref(n)))
    Lb.rsagpu_algo_destroy(algo)
    Lb.rsagpu_radgen_destroy(rg)
    Lb.rsagpu_domain_destroy(dom)
    t1 = time.perf_counter()
    return k, t1 - t0, pos.nbytes + rad.nbytes + phs.nbytes


def run_learned_step(dim, L, r, seed, learned=True):
    """One run of the FP32 form with the learned subdivision schedule (or the heuristic one)."""
    from rsa_mpi_gb300 import _lib
    from rsa_mpi_gb300 import schedule as S
    _, wb = S.load()
    out = S.run_case(dim, L, [(r, 1.0, 0)], seed,
                     schedule=_lib.RSAGPU_SCHEDULE_LEARNED if learned else _lib.RSAGPU_SCHEDULE_HEURISTIC,
                     weights_bf16=wb if learned else None)
    return out["n"], out["stats"]


def config4_instances(n=4096, seed=1):
    """The batching workload: half 2D, half 3D, r = 0.01, box side log-uniform so that the expected counts
    span 1e3 to 1e6 (2D side in [0.758, 23.97], 3D side in [0.2218, 2.218]); Philox key (seed, instance)."""
    import numpy as np
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        dim = 2 if i < n // 2 else 3
        lo, hi = (0.758, 23.97) if dim == 2 else (0.2218, 2.218)
        s = float(np.exp(rng.uniform(math.log(lo), math.log(hi))))
        out.append((dim, [s] * dim, 0.01, (seed << 32) | i))
    return out


def run_single_instances(inst, form):
    """The instances one after another through the single-instance path: (spheres, device seconds)."""
    from rsa_mpi_gb300.sampler import Algo, Domain, RadiusGenerator
    n, ms = 0, 0.0
    for dim, sup, r, seed in inst:
        rg = RadiusGenerator(dim, [(r, 1.0, 0)], volume=float(math.prod(sup)))
        dom = Domain([0.0] * dim, sup, r)
        a = Algo(dom, rg, 6000)
        a.set_form(form)
        a.proceed(seed)
        ms += a.stats()["ms_total"]
        n += dom.count()
        a.close()
        dom.close()
    return n, ms * 1e-3


def batched_form(rank=0, world=1, dist=None):
    """Config 4 through rsagpu_batch_run, and a 64-instance sample of it run both ways and in both forms.
    With N ranks the 4,096 instances are split over them by partition_instances (balanced by expected sphere
    count, no exchange); each rank runs its shard, and the spheres are summed and the seconds max-reduced."""
    from rsa_mpi_gb300.sampler import batch_run, partition_instances
    inst = config4_instances()
    parts = partition_instances(inst, world)
    res = batch_run([inst[i] for i in parts[rank]], form=1)
    st = res["stats"]
    (seconds,), (total,) = aggregate([float(st["seconds"])], [float(res["counts"].sum())], dist,
                                     "cuda" if dist is not None else "cpu")
    total = int(total)
    sample = inst[::64]
    cmp = {}
    for form, name in ((0, "fp64"), (1, "fp32")):
        batch_run(sample, form=form)  # warm
        r2 = batch_run(sample, form=form)
        n1, s1 = run_single_instances(sample, form)
        cmp[name] = {"batched_s": r2["stats"]["seconds"], "single_s": s1, "spheres": n1,
                     "same_counts": int(r2["counts"].sum()) == n1}
    base = cmp["fp64"]["spheres"] / cmp["fp64"]["single_s"]
    return {"workload": "4096 instances, half 2D / half 3D, r=0.01, log-uniform box sides, FP32 form",
            "spheres_per_s": total / seconds, "seconds": seconds, "spheres": total,
            "shards": world, "instances_per_shard": [len(p) for p in parts],
            "waves": st["waves"], "rounds": st["rounds"], "launches": st["launches"], "block_shapes": st["block"],
            "sample_every_64th": cmp,
            "speedup_vs_fp64": (cmp["fp32"]["spheres"] / cmp["fp32"]["batched_s"]) / base,
            "speedup_vs_fp64_note": "sample of 64 instances: batched FP32 vs the single-instance plain FP64 form, "
                                    "one instance after another"}


def precision_form():
    """Config 3 (3D unit cube, radii 0.004 / 0.002 / 0.001 at volume fractions 0.20 / 0.10 / 0.05, seed 1) in the
    plain FP64 form and the FP32 guard-band form: the same spheres (count and centre checksum), the FP64 retests."""
    import numpy as np
    from rsa_mpi_gb300.sampler import Algo, Domain, RadiusGenerator, sphere_checksum
    classes = [(0.004, 0.20, 0), (0.002, 0.10, 0), (0.001, 0.05, 0)]
    out = {}
    for form in (0, 1):
        rg = RadiusGenerator(3, classes, volume=1.0)
        dom = Domain([0.0] * 3, [1.0] * 3, 0.004)
        a = Algo(dom, rg, 6000)
        a.set_form(form)
        a.proceed(1)
        st = a.stats()
        pos, rad, _ = dom.arrays()
        out[form] = {"spheres": int(len(rad)), "ms": st["ms_total"], "retests": st["retests"],
                     "per_class": [int(np.count_nonzero(rad == r)) for r, _, _ in classes],
                     "checksum": sphere_checksum(pos), "maximal": st["maximal"]}
        a.close()
        dom.close()
    return {"workload": "3D unit cube, radii 0.004/0.002/0.001, fractions 0.20/0.10/0.05, seed 1",
            "fp64": out[0], "fp32_guard": out[1],
            "same_spheres": out[0]["checksum"] == out[1]["checksum"] and out[0]["spheres"] == out[1]["spheres"],
            "spheres_per_s_fp64": out[0]["spheres"] / (out[0]["ms"] * 1e-3),
            "spheres_per_s_fp32_guard": out[1]["spheres"] / (out[1]["ms"] * 1e-3),
            "speedup_vs_fp64": out[0]["ms"] / out[1]["ms"]}


def cpu_sample(dim, L, r, seed):
    from oracle import oracle as O
    t0 = time.perf_counter()
    o = O.Oracle(dim, [0.0] * dim, L, [(r, 1.0, 0)])
    o.proceed(seed)
    n = len(o.spheres()[1])
    return n, time.perf_counter() - t0


def _cpu_worker(args):
    dim, L, r, seed = args
    return cpu_sample(dim, L, r, seed)


def reference_arm(args):
    rank, world, _ = env_rank()
    if rank != 0:
        return 0
    import multiprocessing as mp
    from oracle import oracle as O
    O.build()
    cores = os.cpu_count() or 1
    dim, L, r, seed = CPU_SAMPLE
    ctx = mp.get_context("spawn")
    vals = []
    with ctx.Pool(cores) as pool:
        for _ in range(1 if args.warmup > 0 else 0):
            pool.map(_cpu_worker, [(dim, L, r, seed + i) for i in range(cores)])
        step_ms = []
        for s in range(args.steps):
            t0 = time.perf_counter()
            res = pool.map(_cpu_worker, [(dim, L, r, seed + 1000 * s + i) for i in range(cores)])
            el = time.perf_counter() - t0
            vals.append(sum(n for n, _ in res) / el)
            step_ms.append(el * 1e3)
    value = statistics.median(vals)
    wl = WORKLOADS[args.workload]
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "spheres/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": statistics.median(step_ms),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": wl[4], "cpu_sample": "3D periodic box of side 0.2 (1/125 of the unit cube), r=0.002, "
                   f"one instance per core ({cores}), seeds 1000*step+i"},
        "cpu_baseline": {"value": value, "unit": "spheres/s", "cores": cores, "kind": "port",
                         "sample": f"{cores} concurrent instances of the 3D box-0.2 r=0.002 case",
                         "calibration": REFERENCE_CALIBRATION},
        "e2e": {"value": value, "unit": "spheres/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def idle_report(args):
    """GPU busy and idle time (the union of the kernel, memcpy and memset intervals of every stream, and the gaps
    between them) over one run of the workload and one batched run of config 4, each after a warm-up run.  The
    gaps are where the GPU waited on the host: launch latency and the round loop's readbacks.  Records come from
    CUPTI (rsa_mpi_gb300/csrc/activity.cpp), which adds its own small overhead: these runs are not bench values."""
    import ctypes as C
    import torch
    from rsa_mpi_gb300 import build as B
    B.build()
    so = B.build_activity()
    if so is None:
        print(json.dumps({"gpu_idle": None, "why": "no CUPTI in this CUDA toolkit"}))
        return
    act = C.CDLL(so)
    act.rsa_activity_stop.argtypes = [C.POINTER(C.c_double)]
    from rsa_mpi_gb300.sampler import batch_run

    def measure(fn):
        torch.cuda.synchronize()
        rc = act.rsa_activity_start()
        if rc != 0:
            return {"error": f"CUPTI error {rc}"}
        extra = fn()
        torch.cuda.synchronize()
        o = (C.c_double * 8)()
        act.rsa_activity_stop(o)
        span, busy = o[1], o[2]
        return {"records": int(o[0]), "span_ms": span * 1e-6, "busy_ms": busy * 1e-6, "idle_ms": (span - busy) * 1e-6,
                "idle_frac": (span - busy) / span if span else None, "gaps": int(o[3]),
                "gap_median_us": o[4] * 1e-3, "gap_p99_us": o[5] * 1e-3, "gap_max_us": o[6] * 1e-3,
                "gaps_over_10us_ms": o[7] * 1e-6, **extra}

    dim, L, r, seed, desc = WORKLOADS[args.workload]
    run_gpu_step(dim, L, r, seed, args.form)

    def one():
        n, st, _, _, _ = run_gpu_step(dim, L, r, seed, args.form)
        return {"spheres": int(n), "proceed_ms": st["ms_total"], "rounds": st["rounds"]}

    inst = config4_instances()
    batch_run(inst[::16], form=1)

    def batched():
        res = batch_run(inst, form=1)
        st = res["stats"]
        return {"instances": len(inst), "seconds": st["seconds"], "launches": st["launches"],
                "rounds": st["rounds"], "waves": st["waves"]}

    print(json.dumps({"gpu_idle": {args.workload: {"workload": desc, **measure(one)},
                                   "config4 (batched)": measure(batched)}}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="config2", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--form", type=int, default=1, choices=[0, 1], help="0 = plain FP64, 1 = FP32 + guard band")
    ap.add_argument("--no-forms", action="store_true", help="skip the per-form comparison runs")
    ap.add_argument("--idle", action="store_true",
                    help="only report the GPU's busy and idle time over one run of the workload and of config 4 "
                         "(CUPTI activity records), one JSON line")
    args = ap.parse_args()
    if args.impl == "reference":
        return reference_arm(args)
    if args.idle:
        return idle_report(args)

    rank, world, local = env_rank()
    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from rsa_mpi_gb300 import build as B
    B.build()
    from rsa_mpi_gb300.sampler import kernel_launches

    dim, L, r, seed0, desc = WORKLOADS[args.workload]
    seed = seed0 + rank  # each rank samples an independent instance (replicas)
    for _ in range(args.warmup):
        run_gpu_step(dim, L, r, seed, args.form)

    def barrier():
        torch.cuda.synchronize()
        if dist:
            dist.barrier()

    launches0 = kernel_launches()
    barrier()
    spheres, dev_ms, wall = 0, 0.0, 0.0
    mask_ms, mask_bytes, mask_vox = [], [], []
    stats = None
    with ClockSampler(local) as clocks:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            n, st, ms, by, vx = run_gpu_step(dim, L, r, seed, args.form)
            spheres += n
            dev_ms += st["ms_total"]
            mask_ms += list(ms)
            mask_bytes += list(by)
            mask_vox += list(vx)
            stats = st
        barrier()
        wall = time.perf_counter() - t0
    launches = kernel_launches() - launches0

    # the other forms on the same GPU, one run each (outside the timed region)
    forms = {}
    if not args.no_forms:
        primary = {"spheres_per_s": spheres / (dev_ms * 1e-3), "ms": dev_ms / args.steps, "retests": stats["retests"]}
        forms[FORM_NAMES[args.form]] = primary
        other = 1 - args.form
        # the same spheres, by an exact centre checksum (one more run of the timed form, and the other form)
        n1, _, _, _, _, sum1 = run_gpu_step(dim, L, r, seed, args.form, checksum=True)
        n2, st2, _, _, _, sum2 = run_gpu_step(dim, L, r, seed, other, checksum=True)
        primary["checksum"] = sum1
        forms[FORM_NAMES[other]] = {"spheres_per_s": n2 / (st2["ms_total"] * 1e-3), "ms": st2["ms_total"],
                                    "retests": st2["retests"], "checksum": sum2,
                                    "same_spheres": n2 == n1 and sum2 == sum1}
        base = forms[FORM_NAMES[0]]["spheres_per_s"]
        for v in forms.values():
            v["speedup_vs_fp64"] = v["spheres_per_s"] / base
        # learned subdivision schedule (FP32 form), on this workload and on the 4D r = 0.02 hypercube
        nl, stl = run_learned_step(dim, L, r, seed, True)
        learned = {"spheres_per_s": nl / (stl["ms_total"] * 1e-3), "ms": stl["ms_total"], "rounds": stl["rounds"],
                   "refinements": stl["refinements"], "spheres": nl}
        learned["speedup_vs_fp64"] = learned["spheres_per_s"] / base
        h4 = min((run_learned_step(4, [1.0] * 4, 0.02, 5, False) for _ in range(3)), key=lambda t: t[1]["ms_total"])
        l4 = min((run_learned_step(4, [1.0] * 4, 0.02, 5, True) for _ in range(3)), key=lambda t: t[1]["ms_total"])
        learned["4D r=0.02 (held out)"] = {"heuristic_ms": h4[1]["ms_total"], "learned_ms": l4[1]["ms_total"],
                                           "heuristic_rounds": h4[1]["rounds"], "learned_rounds": l4[1]["rounds"],
                                           "heuristic_spheres": h4[0], "learned_spheres": l4[0]}
        forms["learned schedule (FP32 form)"] = learned
        forms["FP32 guard band, polydisperse (config 3)"] = precision_form()
        forms["batched (config 4)"] = batched_form(rank, world, dist)

    # e2e through the C ABI, the spheres read into pinned host buffers allocated once (outside the timed region)
    e2e_n, e2e_s, d2h = 0, 0.0, 0
    outs = pinned_outputs(dim, int(spheres // max(1, args.steps)) + 65536)
    for _ in range(max(1, args.steps)):
        k, s, b = run_e2e_step(dim, L, r, seed, args.form, outs)
        e2e_n += k
        e2e_s += s
        d2h = b
    (dev_ms_max, wall_max, e2e_max), (spheres_all, e2e_all) = aggregate(
        [dev_ms, wall, e2e_s], [float(spheres), float(e2e_n)], dist, "cuda")
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return 0

    peak, peak_kind = measured_peaks()
    import numpy as np
    mm = np.asarray(mask_ms)
    mb = np.asarray(mask_bytes)
    achieved = float(mb.sum() / (mm.sum() * 1e-3) / 1e9) if mm.sum() > 0 else 0.0
    # DRAM traffic per launch: bytes per parent voxel measured by ncu (dram__bytes_read.sum +
    # dram__bytes_write.sum) on a smaller case of the same kernel, times this workload's voxels per launch
    traffic_path = os.path.join(ROOT, "profiles", "refine_mask_traffic.json")
    traffic, traffic_note = None, None
    if os.path.exists(traffic_path) and len(mask_vox):
        tj = json.load(open(traffic_path)).get(FORM_TRAFFIC[args.form], {})
        if tj.get("bytes_per_voxel"):
            traffic = float(tj["bytes_per_voxel"]) * float(np.mean(mask_vox))
            traffic_note = tj.get("note")
    line = {
        "metric": METRIC,
        "value": spheres_all / (dev_ms_max * 1e-3),
        "unit": "spheres/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": dev_ms_max / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64" if args.form == 0 else "f32/f64",
        "data": "synthetic",
        "config": {"workload": desc, "form": FORM_NAMES[args.form], "spheres_per_step": spheres // max(1, args.steps),
                   "parallelism": f"replicas x{world}", "l2": "working set > L2 (no flush needed)"},
        "wall_ms_per_step": wall_max * 1e3 / args.steps,
        "roofline": {"bound": "hbm", "kernel": FORM_KERNEL[args.form], "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_kind": peak_kind, "traffic": traffic, "traffic_note": traffic_note,
                     "voxels_per_launch": float(np.mean(mask_vox)) if len(mask_vox) else 0.0,
                     "share_of_step": float(mm.sum() / max(dev_ms, 1e-9)),
                     "launches": int(len(mm)), "algorithmic_bytes_per_launch": float(mb.mean()) if len(mb) else 0.0},
        "e2e": {"value": e2e_all / e2e_max, "unit": "spheres/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": int(launches),
        "stats": {k: stats[k] for k in ("rounds", "refinements", "darts", "settle_iterations", "peak_voxels", "final_level",
                                         "maximal", "retests")},
        "forms": forms,
    }
    cs = clocks.summary()
    if cs:
        line["clocks"] = cs
    if not args.no_cpu_baseline:
        n, s = cpu_sample(*CPU_SAMPLE)
        line["cpu_baseline"] = {"value": n / s, "unit": "spheres/s", "cores": 1, "kind": "port",
                                "sample": "3D periodic box of side 0.2 (1/125 of the unit cube), r=0.002, seed 1, "
                                          f"to certified maximality: {n} spheres in {s:.1f} s",
                                "calibration": REFERENCE_CALIBRATION}
    print(json.dumps(line))
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
