"""Learned world screen: the batched simulator labels worlds, an MLP learns to propose them.

The reference screens worlds by sampling parameters uniformly and running each one
(scripts/life_screen.py:143-179, 217-245, 538).  Here the batched engine runs many Lenia worlds
at once and labels each from its own trajectory:

  survives  the mass stays within [0.01, 0.9] of the area at every checkpoint
  moves     the toroidal centroid moves more than R cells over the last `window` steps
  explodes  the mass exceeds 0.9 of the area at some checkpoint

A 16 -> 256 -> 256 -> 3 MLP (BF16, trained by this library's kernels, lenia_mlp_*) learns those
labels from 16 features of the parameters.  To screen, it ranks many candidate parameter sets; the
simulator then runs the top ones and judges them, next to the same number of uniform draws.  A
"non-trivial" world survives and moves.

Parameters follow the batched workload's ranges: R ~ U{8..40}, mu ~ U[0.10, 0.35],
sigma ~ U[0.01, 0.06], dt ~ U[0.05, 0.2], plus 1-3 kernel shells with peaks U[0, 1] (the largest
set to 1).  Every draw is unit_f(rand3(i, j, seed)).
"""
import ctypes
import json
import math
import time
from dataclasses import dataclass
from typing import Dict, List, Optional

import numpy as np

from . import _lib
from ._lib import check, fptr
from .program import Kernel, Seed, World
from .sim import Sim

NFEAT = 16


def _pcg(v):
    """program.rs:140-144 on numpy uint64 arrays holding 32-bit values."""
    s = (v * np.uint64(747796405) + np.uint64(2891336453)) & np.uint64(0xFFFFFFFF)
    w = (((s >> ((s >> np.uint64(28)) + np.uint64(4))) ^ s) * np.uint64(277803737)) & np.uint64(0xFFFFFFFF)
    return ((w >> np.uint64(22)) ^ w) & np.uint64(0xFFFFFFFF)


def rand3_array(a, b, c):
    a = np.asarray(a, np.uint64)
    return _pcg(_pcg(_pcg(a) ^ np.uint64(b)) ^ np.uint64(c))


def unit_f_array(r):
    return r.astype(np.float32) * np.float32(1.0 / 4294967296.0)


def sample_params(n: int, seed: int, offset: int = 0) -> Dict[str, np.ndarray]:
    """Parameter set j (j = offset + i) from unit_f(rand3(j, field, seed))."""
    j = np.arange(offset, offset + n, dtype=np.uint64)
    R = (8 + rand3_array(j, 0, seed) % np.uint64(33)).astype(np.float32)
    mu = (0.10 + 0.25 * unit_f_array(rand3_array(j, 1, seed))).astype(np.float32)
    sigma = (0.01 + 0.05 * unit_f_array(rand3_array(j, 2, seed))).astype(np.float32)
    dt = (0.05 + 0.15 * unit_f_array(rand3_array(j, 3, seed))).astype(np.float32)
    nsh = (1 + rand3_array(j, 4, seed) % np.uint64(3)).astype(np.int32)
    beta = np.stack([unit_f_array(rand3_array(j, 5 + s, seed)) for s in range(3)], axis=1)
    beta = np.where(np.arange(3)[None, :] < nsh[:, None], beta, 0.0).astype(np.float32)
    beta /= np.maximum(beta.max(1, keepdims=True), 1e-6)
    return {"R": R, "mu": mu, "sigma": sigma, "dt": dt, "nshells": nsh, "beta": beta}


def features(P: Dict[str, np.ndarray]) -> np.ndarray:
    """16 features of the parameters, each scaled to roughly [0, 1]."""
    R, mu, sg, dt, ns, b = P["R"], P["mu"], P["sigma"], P["dt"], P["nshells"], P["beta"]
    f = np.stack([
        (R - 8) / 32, (mu - 0.10) / 0.25, (sg - 0.01) / 0.05, (dt - 0.05) / 0.15,
        (ns - 1) / 2.0, b[:, 0], b[:, 1], b[:, 2],
        np.clip(mu / sg / 35.0, 0, 1), (np.log(sg) - math.log(0.01)) / math.log(6.0),
        np.clip(dt / sg / 20.0, 0, 1), np.clip(R * sg / 2.4, 0, 1),
        np.clip((mu - 0.5 * sg) / 0.35, 0, 1), np.clip((mu + 2 * sg) / 0.47, 0, 1),
        b[:, :3].sum(1) / 3.0, np.clip(dt * R / 8.0, 0, 1),
    ], axis=1).astype(np.float32)
    assert f.shape[1] == NFEAT
    return f


def worlds_for(P: Dict[str, np.ndarray], side: int) -> List[World]:
    out = []
    q = side // 4
    for i in range(len(P["R"])):
        ns = int(P["nshells"][i])
        k = Kernel(radius=float(P["R"][i]), beta=[float(x) for x in P["beta"][i, :ns]], mu=float(P["mu"][i]),
                   sigma=float(P["sigma"][i]))
        out.append(World(side, side, [k], dt=float(P["dt"][i]), id="screen_%d" % i,
                         seed=Seed("patches", [(q, q, side // 2, side // 2)])))
    return out


def _torus_shift(a, b, n):
    d = np.abs(a - b) % n
    return np.minimum(d, n - d)


def simulate_labels(P: Dict[str, np.ndarray], side: int = 256, steps: int = 2000, every: int = 100,
                    window: int = 500, chunk: int = 4096, path: str = "fp32", seed_base: int = 0) -> Dict:
    """Run every world for `steps` steps in batches of `chunk`; label it from its trajectory."""
    n = len(P["R"])
    area = float(side * side)
    labels = np.zeros((n, 3), np.float32)
    t0 = time.perf_counter()
    gpu_ms = 0.0
    window = min(window, steps)
    for c0 in range(0, n, chunk):
        idx = np.arange(c0, min(n, c0 + chunk))
        sub = {k: v[idx] for k, v in P.items()}
        worlds = worlds_for(sub, side)
        with Sim(worlds, seed=0, path=path) as sim:
            for j, w in enumerate(worlds):
                sim.seed_patches(j, seed_base + int(idx[j]), w.seed.patches)
            ok = np.ones(len(idx), bool)
            boom = np.zeros(len(idx), bool)
            # checkpoints every `every` steps, plus the start of the movement window
            marks = sorted(set(range(every, steps + 1, every)) | {steps - window} - {0})
            start = sim.stats()
            mark = start[:, 1:3].copy()
            done = 0
            for cp in marks:
                gpu_ms += sim.step_timed(cp - done)
                done = cp
                st = sim.stats()
                frac = st[:, 0] / area
                ok &= (frac >= 0.01) & (frac <= 0.9)
                boom |= frac > 0.9
                if cp == steps - window:
                    mark = st[:, 1:3].copy()
            st = sim.stats()
            shift = np.hypot(_torus_shift(st[:, 1], mark[:, 0], side), _torus_shift(st[:, 2], mark[:, 1], side))
            labels[idx, 0] = ok
            labels[idx, 1] = ok & (shift > sub["R"])
            labels[idx, 2] = boom
    return {"labels": labels, "seconds": time.perf_counter() - t0, "gpu_ms": gpu_ms,
            "cell_updates": float(n) * side * side * steps}


class Proposer:
    """The MLP through the C ABI (lenia_mlp_*)."""

    def __init__(self, seed: int = 1, max_batch: int = 4096):
        self.L = _lib.load()
        h = ctypes.c_void_p()
        check(self.L.lenia_mlp_create(seed, max_batch, ctypes.byref(h)), None)
        self.h = h
        self.max_batch = max_batch
        c = ctypes.c_uint32()
        self.L.lenia_mlp_param_count(ctypes.byref(c))
        self.nparam = int(c.value)

    def close(self):
        if self.h:
            self.L.lenia_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self) -> np.ndarray:
        p = np.zeros(self.nparam, np.float32)
        check(self.L.lenia_mlp_get_params(self.h, fptr(p), p.size), None)
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        check(self.L.lenia_mlp_set_params(self.h, fptr(p), p.size), None)

    def gradients(self, x, y):
        x = np.ascontiguousarray(x, np.float32)
        y = np.ascontiguousarray(y, np.float32)
        g = np.zeros(self.nparam, np.float32)
        loss = ctypes.c_float()
        check(self.L.lenia_mlp_gradients(self.h, fptr(x), fptr(y), len(x), fptr(g), ctypes.byref(loss)), None)
        return float(loss.value), g

    def train_step(self, x, y, lr):
        x = np.ascontiguousarray(x, np.float32)
        y = np.ascontiguousarray(y, np.float32)
        loss = ctypes.c_float()
        check(self.L.lenia_mlp_train_step(self.h, fptr(x), fptr(y), len(x), float(lr), ctypes.byref(loss)), None)
        return float(loss.value)

    def fit(self, X, Y, epochs: int = 30, batch: int = 1024, lr: float = 2e-3, seed: int = 0):
        rng = np.random.default_rng(seed)
        hist = []
        for e in range(epochs):
            order = rng.permutation(len(X))
            losses = [self.train_step(X[order[i:i + batch]], Y[order[i:i + batch]], lr)
                      for i in range(0, len(X) - batch + 1, batch)]
            hist.append(float(np.mean(losses)))
        return hist

    def predict(self, X) -> np.ndarray:
        X = np.ascontiguousarray(X, np.float32)
        out = np.zeros((len(X), 3), np.float32)
        check(self.L.lenia_mlp_predict(self.h, fptr(X), len(X), fptr(out)), None)
        return out


def score(probs: np.ndarray) -> np.ndarray:
    """Rank by the chance of a surviving, moving, non-exploding world."""
    return probs[:, 1] * (1.0 - probs[:, 2])


@dataclass
class ScreenConfig:
    train_worlds: int = 50000
    side: int = 256
    steps: int = 2000
    every: int = 100
    window: int = 500
    candidates: int = 1_000_000
    top: int = 4096
    epochs: int = 40
    seed: int = 5


def run(cfg: ScreenConfig, path: str = "fp32", log=print) -> Dict:
    """Generate labelled worlds, train, rank candidates, and judge top-k against uniform draws."""
    P = sample_params(cfg.train_worlds, cfg.seed)
    data = simulate_labels(P, cfg.side, cfg.steps, cfg.every, cfg.window, path=path)
    X, Y = features(P), data["labels"]
    log("training data: %d worlds, %.1f s (%.3e cell-updates/s on the GPU); rates survive %.3f move %.3f explode %.3f"
        % (len(X), data["seconds"], data["cell_updates"] / (data["gpu_ms"] * 1e-3), Y[:, 0].mean(), Y[:, 1].mean(),
           Y[:, 2].mean()))
    mlp = Proposer(seed=cfg.seed)
    t0 = time.perf_counter()
    hist = mlp.fit(X, Y, epochs=cfg.epochs)
    t_train = time.perf_counter() - t0
    C = sample_params(cfg.candidates, cfg.seed + 1)
    t0 = time.perf_counter()
    probs = mlp.predict(features(C))
    t_rank = time.perf_counter() - t0
    top = np.argsort(-score(probs))[: cfg.top]
    chosen = {k: v[top] for k, v in C.items()}
    uni = sample_params(cfg.top, cfg.seed + 2)
    judged_l = simulate_labels(chosen, cfg.side, cfg.steps, cfg.every, cfg.window, path=path, seed_base=10_000_000)
    judged_u = simulate_labels(uni, cfg.side, cfg.steps, cfg.every, cfg.window, path=path, seed_base=20_000_000)
    nl = judged_l["labels"]
    nu = judged_u["labels"]
    good_l = int(nl[:, 1].sum())
    good_u = int(nu[:, 1].sum())
    # per GPU-hour, two ways.  Amortised: the learned screen pays for its ranking on top of the
    # simulations it judges (the cost once a trained model is reused).  All-in: it also pays for the
    # simulations that labelled its training set and for its training.
    hours_l = (judged_l["gpu_ms"] * 1e-3 + t_rank) / 3600.0
    hours_u = judged_u["gpu_ms"] * 1e-3 / 3600.0
    fixed_s = data["gpu_ms"] * 1e-3 + t_train
    hours_l_all = hours_l + fixed_s / 3600.0
    rep = {
        "train_worlds": cfg.train_worlds, "side": cfg.side, "steps": cfg.steps, "candidates": cfg.candidates,
        "top": cfg.top, "train_loss_first_last": [hist[0], hist[-1]], "train_seconds": t_train,
        "rank_seconds": t_rank, "label_rates_train": Y.mean(0).tolist(),
        "learned": {"survive": int(nl[:, 0].sum()), "nontrivial": good_l, "explode": int(nl[:, 2].sum()),
                    "gpu_hours": hours_l, "nontrivial_per_gpu_hour": good_l / hours_l if hours_l else None},
        "uniform": {"survive": int(nu[:, 0].sum()), "nontrivial": good_u, "explode": int(nu[:, 2].sum()),
                    "gpu_hours": hours_u, "nontrivial_per_gpu_hour": good_u / hours_u if hours_u else None},
    }
    rep["gain_nontrivial_per_gpu_hour"] = (rep["learned"]["nontrivial_per_gpu_hour"] /
                                           rep["uniform"]["nontrivial_per_gpu_hour"]
                                           if good_u else None)
    rep["all_in"] = all_in_accounting(good_l, good_u, cfg.top, hours_l * 3600.0, hours_u * 3600.0, fixed_s,
                                      data["gpu_ms"] * 1e-3, t_train)
    rep["label_positives_train"] = {"survive": int(Y[:, 0].sum()), "move": int(Y[:, 1].sum()),
                                    "explode": int(Y[:, 2].sum())}
    if int(Y[:, 2].sum()) == 0:
        rep["explode_head"] = ("untrained: no world in the training ranges exploded (mass above 0.9 of the area), "
                               "so the head only learns to predict 0; the ranking score's (1 - p_explode) is then ~1")
    mlp.close()
    return rep


def all_in_accounting(good_l, good_u, judged, judge_s_l, judge_s_u, fixed_s, data_s, train_s):
    """The learned screen charged in full: labelling its training set (simulator GPU time) and training
    it, on top of ranking and judging.  With n worlds judged per trained model, its yield per GPU-hour
    is (good_l / judged) n / (fixed + (judge_s_l / judged) n); the uniform screen's is good_u / judge_s_u.
    Returns the all-in ratio at this run's n and the n at which the learned screen breaks even (1x) and
    reaches 3x (None if it never does: its per-world rate times the uniform cost is below 3x)."""
    rate_l, cost_l = good_l / judged, judge_s_l / judged
    yield_u = good_u / judge_s_u if judge_s_u and good_u else None
    total_l = fixed_s + judge_s_l
    out = {"fixed_seconds": fixed_s, "training_data_gpu_seconds": data_s, "training_seconds": train_s,
           "learned_seconds_all_in": total_l, "nontrivial_per_gpu_hour_all_in": good_l / (total_l / 3600.0),
           "gain_all_in": (good_l / total_l) / yield_u if yield_u else None}
    for name, f in (("break_even_judged_worlds", 1.0), ("judged_worlds_for_3x", 3.0)):
        den = rate_l - f * yield_u * cost_l if yield_u else 0.0
        out[name] = f * yield_u * fixed_s / den if den > 0 else None
    return out


if __name__ == "__main__":
    import argparse
    ap = argparse.ArgumentParser()
    ap.add_argument("--train-worlds", type=int, default=50000)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--candidates", type=int, default=1_000_000)
    ap.add_argument("--top", type=int, default=4096)
    ap.add_argument("--epochs", type=int, default=40)
    ap.add_argument("--out", default=None)
    a = ap.parse_args()
    cfg = ScreenConfig(train_worlds=a.train_worlds, steps=a.steps, candidates=a.candidates, top=a.top, epochs=a.epochs)
    rep = run(cfg)
    print(json.dumps(rep))
    if a.out:
        json.dump(rep, open(a.out, "w"), indent=1)
