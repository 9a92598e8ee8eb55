"""Learned subdivision schedule: data, targets and training of the 16-64-64-2 network.

After every dart pass the sampler decides whether to subdivide the voxels now or to throw another pass at
the current level.  The fixed heuristic subdivides when the pass's miss rate exceeds a threshold.  The
learned schedule asks the network for the predicted remaining time after each action -- y[0] for one
more pass, y[1] for subdividing now -- and takes the smaller; the heuristic stays as the fallback when
no weights are loaded or an output is not finite.

State features (computed by the library after each pass, rsagpu_algo_trace_features):
  0 log2(V + 1)/32              voxels before the pass
  1 level/32                    subdivision level
  2 miss rate of the pass       (darts not accepted, count cap excluded)
  3 miss rate of the previous pass at this level (= 2 on the first pass)
  4 min(passes at this level, 16)/16
  5 log2(darts + 1)/32
  6 log2(accepted + 1)/32
  7 log2(spheres placed + 1)/32
  8 packing fraction so far
  9 D/8
 10 log2(V / grid cells + 1e-9)/32
 11 accepted / (V + 1)
 12 log2(level-0 voxels)/32
 13 voxels kept by the last subdivision / (2^D x voxels before it)  (1 before the first)
 14 heuristic's decision (1 = subdivide)
 15 1 (bias)

Training (fitted Monte Carlo Q values): episodes of small runs (configs 1-3 and their kin) with the
heuristic's decisions flipped at random; for each decision the target of the action taken is the wall
time that followed it until the end of the run (the subdivision itself included), as log2(ms + 0.05)/10;
the other output has no target.  The network is trained on the GPU by rsagpu_mlp_train_step.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _lib
from ._lib import check, lib, ptr
from .sampler import Algo, Domain, RadiusGenerator

NW = 5378
WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "schedule_mlp.npz")

# training cases: (dim, L, classes[(r, phi, phase)]) -- configs 1 to 3 and smaller relatives
TRAIN_CASES = [
    (2, [1.0, 1.0], [(0.005, 1.0, 0)]),
    (2, [1.0, 1.0], [(0.003, 1.0, 0)]),
    (3, [1.0, 1.0, 1.0], [(0.01, 1.0, 0)]),
    (3, [1.0, 1.0, 1.0], [(0.006, 1.0, 0)]),
    (3, [1.0, 1.0, 1.0], [(0.004, 1.0, 0)]),
    (3, [1.0, 1.0, 1.0], [(0.008, 0.20, 0), (0.004, 0.10, 1), (0.002, 0.05, 2)]),
    (3, [1.0, 1.0, 1.0], [(0.003, 1.0, 0)]),
    (3, [0.5, 0.5, 0.5], [(0.002, 1.0, 0)]),
]


def init_weights(seed=0):
    rng = np.random.default_rng(seed)
    w = np.zeros(NW, np.float32)
    o = 0
    for fan_in, n_out in ((16, 64), (64, 64), (64, 2)):
        n = fan_in * n_out
        w[o:o + n] = rng.normal(0, np.sqrt(2.0 / fan_in), n).astype(np.float32)
        o += n + n_out  # biases start at 0
    return w


def to_bf16(w32):
    """Round-to-nearest-even to bf16 bit patterns."""
    u = np.asarray(w32, np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)
    return r


def features_trace(algo: Algo):
    n = C.c_uint64()
    check(lib().rsagpu_algo_trace_features(algo._h, None, None, None, None, 0, C.byref(n)))
    k = n.value
    f = np.zeros((max(k, 1), 16), np.float32)
    a = np.zeros(max(k, 1), np.uint8)
    pm = np.zeros(max(k, 1))
    rm = np.zeros(max(k, 1))
    check(lib().rsagpu_algo_trace_features(algo._h, ptr(f, _lib._f32), ptr(a, _lib._u8), ptr(pm, _lib._d),
                                           ptr(rm, _lib._d), k, C.byref(n)))
    return f[:k], a[:k].astype(bool), pm[:k], rm[:k]


def run_case(dim, L, classes, seed, schedule=_lib.RSAGPU_SCHEDULE_HEURISTIC, weights_bf16=None, eps=0.0,
             form=_lib.RSAGPU_FORM_FP32_GUARD, **sched):
    vol = float(np.prod(L))
    rg = RadiusGenerator(dim, classes, volume=vol)
    dom = Domain([0.0] * dim, L, rg.max_radius)
    algo = Algo(dom, rg, 6000)
    algo.set_form(form, schedule)
    if sched:
        algo.set_schedule(**sched)
    if weights_bf16 is not None:
        algo.set_mlp(weights_bf16)
    if eps > 0:
        check(lib().rsagpu_algo_set_exploration(algo._h, float(eps), int(seed) * 7919 + 1))
    algo.proceed(seed)
    out = dict(stats=algo.stats(), trace=features_trace(algo), n=dom.count(), check=dom.check(),
               fraction=dom.spheres_volume() / vol)
    algo.close()
    dom.close()
    return out


def targets_from_trace(feat, refined, pass_ms, refine_ms):
    """Q target of the action taken at each decision: log2 of the wall time (ms) after it, to the end of the
    run, the decision's own subdivision included (log scale: runs differ by orders of magnitude)."""
    after = np.zeros(len(feat))
    acc = 0.0
    for t in range(len(feat) - 1, -1, -1):
        after[t] = acc + refine_ms[t]
        acc += pass_ms[t] + refine_ms[t]
    tgt = np.full((len(feat), 2), np.nan, np.float32)
    tgt[np.arange(len(feat)), refined.astype(int)] = (np.log2(after + 0.05) / 10).astype(np.float32)
    return tgt


def generate(episodes_per_case=12, seed0=100, eps_choices=(0.1, 0.2, 0.3, 0.5)):
    X, T = [], []
    k = 0
    for case in TRAIN_CASES:
        for e in range(episodes_per_case):
            eps = eps_choices[e % len(eps_choices)]
            out = run_case(*case, seed=seed0 + k, schedule=_lib.RSAGPU_SCHEDULE_LEARNED, eps=eps)
            k += 1
            f, a, pm, rm = out["trace"]
            if len(f) == 0:
                continue
            X.append(f)
            T.append(targets_from_trace(f, a, pm, rm))
    return np.concatenate(X), np.concatenate(T)


def train_step(master, wb, X, T, lr):
    loss = C.c_float()
    grad = np.zeros(NW, np.float32)
    check(lib().rsagpu_mlp_train_step(ptr(master, _lib._f32), ptr(wb, _lib._u16), ptr(X, _lib._f32),
                                      ptr(T, _lib._f32), len(X), float(lr), C.byref(loss), ptr(grad, _lib._f32)))
    return loss.value, grad


def forward(wb, X):
    X = np.ascontiguousarray(X, np.float32)
    Y = np.zeros((len(X), 2), np.float32)
    check(lib().rsagpu_mlp_forward(ptr(np.ascontiguousarray(wb, np.uint16), _lib._u16), ptr(X, _lib._f32), len(X),
                                   ptr(Y, _lib._f32)))
    return Y


def train(X, T, steps=3000, lr=0.05, seed=0, log_every=500):
    master = init_weights(seed)
    wb = to_bf16(master)
    X = np.ascontiguousarray(X, np.float32)
    T = np.ascontiguousarray(T, np.float32)
    losses = []
    for s in range(steps):
        loss, _ = train_step(master, wb, X, T, lr * (0.3 if s > steps * 0.7 else 1.0))
        losses.append(loss)
        if log_every and s % log_every == 0:
            print(f"step {s} loss {loss:.5f}", flush=True)
    return master, wb, np.asarray(losses)


def save(master, wb, path=WEIGHTS, **meta):
    np.savez(path, master=master, bf16=wb, **meta)


def load(path=WEIGHTS):
    z = np.load(path)
    return z["master"], z["bf16"]


if __name__ == "__main__":
    import json
    import sys
    import time
    t0 = time.time()
    X, T = generate()
    print(f"samples {len(X)} in {time.time() - t0:.1f}s", flush=True)
    master, wb, losses = train(X, T)
    out = sys.argv[1] if len(sys.argv) > 1 else WEIGHTS
    save(master, wb, out, final_loss=losses[-1], samples=len(X))
    print(json.dumps({"samples": int(len(X)), "loss0": float(losses[0]), "loss": float(losses[-1])}))
