"""The synthetic benchmark workloads, built deterministically from the PCG hash.

Every random draw is ``unit_f(rand3(a, b, c))`` (program.rs:140-147) so that the workloads are
identical on every machine.  Configurations:

  1. ``single_256``     one 256x256 world, R=13, beta=[1], mu=.15, sigma=.015, dt=.1, seed 0,
                        U[0,1] in the centred 64x64 patch
  2. ``single_4096``    one 4096x4096 world, R=52, beta=[1,.5,.25], mu=.26, sigma=.036, dt=.05,
                        seed 1, 16 random 256x256 patches
  3. ``batched(n)``     n worlds, sides from {128,...,1024}, per-world R~U{8..40},
                        mu~U[.10,.35], sigma~U[.01,.06], dt~U[.05,.2], centred patch of 25% area
  4. ``multichannel``   3 channels at 1024x1024, 9 kernels (every src->dst pair), R~U{10..30},
                        1-3 shells with peaks U[0,1], mu~U[.1,.4], sigma~U[.01,.05], weights U[0,1]
                        normalised per target channel, dt=.2, U[0,1] everywhere
"""
from typing import List, Tuple

from .program import Kernel, Seed, World, rand3, unit_f
from ._lib import RULE_LENIA, SHAPE_LENIA

BATCH_SIDES = (128, 192, 256, 384, 512, 768, 1024)


def single_256() -> World:
    w = World(256, 256, [Kernel(SHAPE_LENIA, 13.0, [1.0], mu=0.15, sigma=0.015)], dt=0.1, rule=RULE_LENIA,
              id="single_256", seed=Seed("patches", [(96, 96, 64, 64)]))
    return w


SEED_256 = 0


def single_4096_patches() -> List[Tuple[int, int, int, int]]:
    return [(rand3(i, 0, 1) % 3840, rand3(i, 1, 1) % 3840, 256, 256) for i in range(16)]


def single_4096() -> World:
    return World(4096, 4096, [Kernel(SHAPE_LENIA, 52.0, [1.0, 0.5, 0.25], mu=0.26, sigma=0.036)], dt=0.05,
                 rule=RULE_LENIA, id="single_4096", seed=Seed("patches", single_4096_patches()))


SEED_4096 = 1


def batched_world(i: int) -> World:
    """World i of the batched workload; its parameters come from rand3(i, k, 3)."""
    side = BATCH_SIDES[rand3(i, 0, 3) % len(BATCH_SIDES)]
    R = 8 + rand3(i, 1, 3) % 33
    mu = 0.10 + 0.25 * unit_f(rand3(i, 2, 3))
    sigma = 0.01 + 0.05 * unit_f(rand3(i, 3, 3))
    dt = 0.05 + 0.15 * unit_f(rand3(i, 4, 3))
    q = side // 4
    return World(side, side, [Kernel(SHAPE_LENIA, float(R), [1.0], mu=mu, sigma=sigma)], dt=dt, rule=RULE_LENIA,
                 id="batched_%d" % i, seed=Seed("patches", [(q, q, side // 2, side // 2)]))


def batched(n: int = 384) -> List[World]:
    return [batched_world(i) for i in range(n)]


def multichannel() -> World:
    kernels = []
    raw_w = []
    k = 0
    for src in range(3):
        for dst in range(3):
            R = 10 + rand3(k, 0, 4) % 21
            nsh = 1 + rand3(k, 1, 4) % 3
            beta = [unit_f(rand3(k, 10 + j, 4)) for j in range(nsh)]
            if max(beta) <= 0.0:
                beta[0] = 1.0
            mu = 0.1 + 0.3 * unit_f(rand3(k, 2, 4))
            sigma = 0.01 + 0.04 * unit_f(rand3(k, 3, 4))
            raw_w.append(unit_f(rand3(k, 4, 4)))
            kernels.append(Kernel(SHAPE_LENIA, float(R), beta, src=src, dst=dst, mu=mu, sigma=sigma))
            k += 1
    for dst in range(3):
        idx = [i for i, kk in enumerate(kernels) if kk.dst == dst]
        tot = sum(raw_w[i] for i in idx) or 1.0
        for i in idx:
            kernels[i].weight = raw_w[i] / tot
    return World(1024, 1024, kernels, channels=3, dt=0.2, rule=RULE_LENIA, id="multichannel",
                 seed=Seed("patches", [(0, 0, 1024, 1024)]))


SEED_MULTI = 4
