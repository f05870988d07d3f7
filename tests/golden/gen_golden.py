"""Generate the golden fixtures under tests/golden/ from the reference project's own sources.

Run where the reference checkout is available: pass its path as the first argument, or set
AUTO_REFERENCE to it (there is no default).  The reference is Rust + WGSL and cannot run here, so this script restates in pure
Python/numpy -- independently of oracle/lenia_oracle.c -- exactly what its one Lenia test does:

* crates/auto-core/src/automata/spectral.rs:287       the Orbium table (u8, 20x20)
* crates/auto-core/src/automata/spectral.rs:313-335   tile seeding: rand3(tx, ty, seed), even -> creature,
                                                      quarter turn from (r >> 8) & 3
* crates/auto-core/src/program.rs:140-147             pcg / rand3 / unit_f
* crates/auto-core/tests/automata.rs:302-314          the first seed in 1..64 that places an Orbium on 128x64
* crates/auto-core/tests/automata.rs:316-355          f64 direct torus convolution + Lenia growth, one step

Outputs (small, committed):
  orbium.npy              uint8 (20, 20)
  lenia_128x64.npz        seed, state0 (f32), want_direct (f32, one step), tolerance 2e-3
  pcg_vectors.npz         rand3 / unit_f known answers on a grid of inputs
"""
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
M32 = 0xFFFFFFFF


def pcg(v):
    s = (v * 747796405 + 2891336453) & M32
    w = (((s >> ((s >> 28) + 4)) ^ s) * 277803737) & M32
    return ((w >> 22) ^ w) & M32


def rand3(a, b, c):
    return pcg(pcg(pcg(a) ^ b) ^ c)


def unit_f(r):
    return np.float32(np.float32(r) * np.float32(1.0 / 4294967296.0))


def read_orbium(ref_root):
    src = open(os.path.join(ref_root, "crates/auto-core/src/automata/spectral.rs")).read()
    m = re.search(r'const ORBIUM: &str = "([0-9u,]+)";', src)
    vals = [int(t.rstrip("u")) for t in m.group(1).split(",")]
    assert len(vals) == 400
    return np.array(vals, np.uint8).reshape(20, 20)


def seed_tiles(w, h, seed, orbium, spacing=64):
    out = np.zeros((h, w), np.float32)
    for y in range(h):
        for x in range(w):
            r = rand3(x // spacing, y // spacing, seed)
            if r & 1:
                continue
            px, py = x % spacing, y % spacing
            if px >= 20 or py >= 20:
                continue
            ix, iy = px, py
            turn = (r >> 8) & 3
            if turn == 1:
                ix, iy = py, 19 - px
            elif turn == 2:
                ix, iy = 19 - px, 19 - py
            elif turn == 3:
                ix, iy = 19 - py, px
            out[y, x] = np.float32(orbium[iy, ix]) / np.float32(255.0)
    return out


def direct_step(start, radius=13.0, reach=14, mu=0.15, sigma=0.015, dt=0.1):
    h, w = start.shape
    dy, dx = np.mgrid[-reach:reach + 1, -reach:reach + 1]
    q = np.sqrt((dx * dx + dy * dy).astype(np.float64)) / radius
    core = np.zeros_like(q)
    m = (q > 0) & (q < 1)
    core[m] = np.exp(4.0 - 1.0 / (q[m] * (1.0 - q[m])))
    total = core.sum()
    u = np.zeros((h, w), np.float64)
    s64 = start.astype(np.float64)
    for j in range(2 * reach + 1):
        for i in range(2 * reach + 1):
            k = core[j, i]
            if k > 0.0:
                # u[y, x] += k * start[(y + dy) mod h, (x + dx) mod w]
                u += k * np.roll(np.roll(s64, -(j - reach), axis=0), -(i - reach), axis=1)
    d = (u / total - mu) / sigma
    g = 2.0 * np.exp(-0.5 * d * d) - 1.0
    return np.clip(s64 + dt * g, 0.0, 1.0).astype(np.float32)


def main(ref_root):
    orbium = read_orbium(ref_root)
    np.save(os.path.join(HERE, "orbium.npy"), orbium)
    w, h = 128, 64
    for seed in range(1, 64):
        state0 = seed_tiles(w, h, seed, orbium)
        if (state0 > 0).any():
            break
    want = direct_step(state0)
    np.savez_compressed(os.path.join(HERE, "lenia_128x64.npz"), seed=np.uint32(seed), state0=state0,
                        want_direct=want, tolerance=np.float32(0.002))
    a = np.arange(0, 4096, 97, dtype=np.uint64)
    triples = np.array([(int(x), int(x * 7 + 3) & M32, int(x ^ 0xDEADBEEF)) for x in a], np.uint32)
    r3 = np.array([rand3(int(t[0]), int(t[1]), int(t[2])) for t in triples], np.uint32)
    uf = np.array([unit_f(int(r)) for r in r3], np.float32)
    np.savez_compressed(os.path.join(HERE, "pcg_vectors.npz"), triples=triples, rand3=r3, unit_f=uf)
    print("seed", seed, "mass", float(state0.sum()), "want mass", float(want.sum()))


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("AUTO_REFERENCE")
    if not ref:
        sys.exit("usage: gen_golden.py REFERENCE_CHECKOUT (or set AUTO_REFERENCE)")
    main(ref)
