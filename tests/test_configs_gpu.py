"""The benchmark configurations at their full size and over their full length, on a GB300, against
the FP64 oracle, teacher-forced: at each checkpoint the engine and the oracle take one step from
the same state (the engine's own state at that point), as the reference's one Lenia test does for
a single step (crates/auto-core/tests/automata.rs:300-362).

Tolerances (per-step max-abs against FP64):
  * FP32 path: 1e-5 on the one-channel configurations, 1e-4 on the 3-channel world
  * BF16x3 tensor-core path (column pass, and with +tc_rows the row pass too): 1e-4, the metric's
    bound
Each checkpoint also reports the world's mass, so a run that has died out (a trivial comparison)
shows as such: the 3-channel configuration does die out, at step 8 in FP64 and on the GPU alike,
which the test asserts.
"""
import numpy as np
import pytest

from auto_gb300 import Sim, configs
from oracle.oracle import fp64_khats, fp64_step

pytestmark = pytest.mark.gpu

TOL = {"fp32": 1e-5, "bf16x3": 1e-4, "bf16x3+tc_rows": 1e-4}


@pytest.fixture(scope="module", autouse=True)
def built():
    from auto_gb300 import native, _lib
    native.build()
    _lib.load()


def split_states(worlds, flat):
    out, off = [], 0
    for w in worlds:
        n = w.channels * w.height * w.width
        out.append(flat[off:off + n].reshape(w.channels, w.height, w.width))
        off += n
    return out


@pytest.fixture(scope="module")
def batched384():
    worlds = configs.batched(384)
    return worlds, [fp64_khats(w) for w in worlds]


@pytest.mark.parametrize("path", ["fp32", "bf16x3", "bf16x3+tc_rows"])
def test_config3_all_384_worlds_at_checkpoints(batched384, path):
    """Configuration 3 whole: all 384 uneven worlds (sides 128..1024, per-world R, mu, sigma, dt) in
    one context, seeded with their 25%-area patches, checked at generations 1, 16 and 64 -- the
    64-step graph the bench replays.  bf16x3+tc_rows runs the row pass on the tensor cores too, where
    it applies (sides 256, 512, 1024)."""
    worlds, khats = batched384
    worst, dead = 0.0, 0
    with Sim(worlds, seed=0, path=path.split("+")[0]) as sim:
        if path.endswith("tc_rows"):
            sim.set_tc_rows(True)
        for i, w in enumerate(worlds):
            sim.seed_patches(i, i, w.seed.patches)
        done = 0
        for cp in (1, 16, 64):
            if cp - 1 > done:
                sim.step(cp - 1 - done)
            before = split_states(worlds, sim.read_states().copy())
            sim.step(1)
            done = cp
            after = split_states(worlds, sim.read_states())
            cp_worst = 0.0
            for i, w in enumerate(worlds):
                err = float(np.abs(after[i] - fp64_step(w, before[i], khats=khats[i])).max())
                assert err < TOL[path], (path, cp, i, w.width, err)
                cp_worst = max(cp_worst, err)
            masses = np.array([a.mean() for a in after])
            dead = int((masses == 0).sum())
            print("config3 %s generation %d: worst per-step max|err| vs FP64 %.3e over 384 worlds; mean mass "
                  "%.4f, worlds died out %d" % (path, cp, cp_worst, masses.mean(), dead))
            worst = max(worst, cp_worst)
    # most worlds are alive at the last checkpoint, so the comparison is not of empty grids
    assert dead < 384 // 2, dead


@pytest.mark.parametrize("path", ["fp32", "bf16x3"])
def test_config2_4096_over_500_steps(path):
    """Configuration 2 whole: the 4096x4096 world (R=52, three shells) run for its 500 steps, checked
    at steps 1, 100, 250 and 500."""
    world = configs.single_4096()
    khats = fp64_khats(world)
    with Sim(world, seed=configs.SEED_4096, path=path) as sim:
        done = 0
        for cp in (1, 100, 250, 500):
            if cp - 1 > done:
                sim.step(cp - 1 - done)
            before = sim.read_state(0)
            sim.step(1)
            done = cp
            got = sim.read_state(0)
            err = float(np.abs(got - fp64_step(world, before, khats=khats)).max())
            mass = float(got.mean())
            print("config2 %s step %d: per-step max|err| vs FP64 %.3e, mean state %.5f" % (path, cp, err, mass))
            assert err < TOL[path], (cp, err)
            assert 0.0 < mass < 1.0, (cp, mass)


def test_config4_multichannel_over_300_steps():
    """Configuration 4 whole: 3 channels at 1024x1024 with 9 kernels and dt = 0.2, checked after every
    one of its first 8 steps and at steps 50, 150 and 300.  From U[0,1] everywhere this world dies
    out: its growth is negative almost everywhere, and every channel reaches exactly 0 at step 8 (the
    FP64 oracle shows the same).  After that U = 0, the growth is -1 and the clamp keeps the state at
    0, so the later checkpoints compare empty grids; they are asserted to be exactly empty."""
    world = configs.multichannel()
    khats = fp64_khats(world)
    with Sim(world, seed=configs.SEED_MULTI) as sim:
        done = 0
        for cp in (1, 2, 3, 4, 5, 6, 7, 8, 50, 150, 300):
            if cp - 1 > done:
                sim.step(cp - 1 - done)
            before = sim.read_state(0)
            sim.step(1)
            done = cp
            got = sim.read_state(0)
            want = fp64_step(world, before, khats=khats)
            err = float(np.abs(got - want).max())
            mass = got.reshape(3, -1).mean(axis=1)
            print("config4 step %d: per-step max|err| vs FP64 %.3e, mean state per channel %s" %
                  (cp, err, " ".join("%.6f" % m for m in mass)))
            assert err < 1e-4, (cp, err)
            if cp >= 8:
                assert not want.any(), cp
            if cp >= 50:
                assert not got.any(), cp
            if cp <= 6:
                assert (mass > 0).all(), (cp, mass)
