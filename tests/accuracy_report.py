"""Accuracy of every step path on every workload against the FP64 oracle (run on a GB300).

For each workload and path it reports:
  per_step   max over steps of max|engine(s_t) - FP64(s_t)|, teacher-forced: both sides step from
             the engine's own state s_t
  vs_ref     the same against the f32 restatement of the reference's step (one-channel,
             power-of-two worlds only: the reference supports nothing else)
  div_100    max|engine^100(s_0) - FP64^100(s_0)| after 100 free-running steps from the same
             start: trajectory divergence, which chaos amplifies; reported, never gated

Usage: python tests/accuracy_report.py [--out profiles/accuracy.md] [--quick]
This is test infrastructure (it runs the oracle), not part of the library.
"""
import argparse
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import auto_gb300 as ag  # noqa: E402
from auto_gb300 import configs  # noqa: E402
from oracle.oracle import RefF32, fp64_khats, fp64_step  # noqa: E402


def seeded(sim, worlds, seeds):
    for i, (w, s) in enumerate(zip(worlds, seeds)):
        sim.seed_patches(i, s, w.seed.patches)


def teacher_forced(worlds, seeds, path, steps, ref=None, skip_first=0):
    """Per-step errors over `steps` steps (after `skip_first` untested steps)."""
    khats = [fp64_khats(w) for w in worlds]
    spectra = [ref.spectra(w) for w in worlds] if ref else None
    worst64 = worst_ref = 0.0
    with ag.Sim(worlds, seed=0, path=path) as sim:
        seeded(sim, worlds, seeds)
        if skip_first:
            sim.step(skip_first)
        prev = [sim.read_state(i) for i in range(len(worlds))]
        for _ in range(steps):
            sim.step(1)
            for i, w in enumerate(worlds):
                got = sim.read_state(i)
                worst64 = max(worst64, float(np.abs(got - fp64_step(w, prev[i], khats=khats[i])).max()))
                if ref:
                    want = ref.step(w, prev[i][0], spectra=spectra[i], threads=1)
                    worst_ref = max(worst_ref, float(np.abs(got[0] - want).max()))
                prev[i] = got
    return worst64, (worst_ref if ref else None)


def divergence(worlds, seeds, path, steps=100):
    out = 0.0
    with ag.Sim(worlds, seed=0, path=path) as sim:
        seeded(sim, worlds, seeds)
        start = [sim.read_state(i) for i in range(len(worlds))]
        sim.step(steps)
        for i, w in enumerate(worlds):
            want = fp64_step(w, start[i], steps=steps)
            out = max(out, float(np.abs(sim.read_state(i) - want).max()))
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=os.path.join(ROOT, "profiles", "accuracy.md"))
    ap.add_argument("--quick", action="store_true")
    a = ap.parse_args()
    ref = RefF32()
    q = a.quick
    cases = [
        ("single_256 (256^2, R=13)", [configs.single_256()], [configs.SEED_256], 100 if q else 1000, True,
         ["fp32", "radix2", "bf16x3", "tf32"]),
        ("single_4096 (4096^2, R=52, 3 shells)", [configs.single_4096()], [configs.SEED_4096], 3 if q else 10, True,
         ["fp32", "radix2", "bf16x3", "tf32"]),
        ("batched (384 worlds, 128..1024)", configs.batched(384), list(range(384)), 1, False,
         ["fp32", "bf16x3", "tf32"]),
        ("multichannel (3 x 1024^2, 9 kernels)", [configs.multichannel()], [configs.SEED_MULTI], 3 if q else 5, False,
         ["fp32", "bf16x3", "tf32"]),
    ]
    rows = []
    for name, worlds, seeds, steps, use_ref, paths in cases:
        div_worlds = worlds if len(worlds) <= 16 else worlds[::24]
        div_seeds = seeds if len(seeds) <= 16 else seeds[::24]
        for path in paths:
            t0 = time.time()
            per_step, vs_ref = teacher_forced(worlds, seeds, path, steps, ref if use_ref else None)
            div = divergence(div_worlds, div_seeds, path, 100)
            rows.append({"workload": name, "path": path, "steps": steps, "per_step": per_step, "vs_ref": vs_ref,
                         "div_100": div, "worlds_in_div": len(div_worlds), "seconds": time.time() - t0})
            print(json.dumps(rows[-1]), flush=True)
    lines = ["# Accuracy against the FP64 oracle", "",
             "Produced on a GB300 by `python tests/accuracy_report.py` (teacher-forced per-step max-abs error;",
             "100-step free-running divergence reported, not gated). Target: per step <= 1e-4 vs FP64; the",
             "reference's own step (restated in f32) within 1e-5 on the workloads it supports.", "",
             "| workload | path | steps checked | per step vs FP64 | per step vs reference f32 step | 100-step divergence |",
             "|---|---|---|---|---|---|"]
    for r in rows:
        lines.append("| %s | %s | %d | %.2e | %s | %.2e (%d worlds) |" % (
            r["workload"], r["path"], r["steps"], r["per_step"],
            "%.2e" % r["vs_ref"] if r["vs_ref"] is not None else "n/a (reference has no such world)",
            r["div_100"], r["worlds_in_div"]))
    os.makedirs(os.path.dirname(a.out), exist_ok=True)
    open(a.out, "w").write("\n".join(lines) + "\n")
    json.dump(rows, open(a.out.replace(".md", ".json"), "w"), indent=1)


if __name__ == "__main__":
    main()
