"""Parity of the CUDA engine with the oracle, through the C ABI (ctypes), on a GB300.

Tolerances:
  * the reference's own test: worst < 2e-3 (tests/automata.rs:361); we also hold 1e-5
  * per step against the f32 restatement of the reference step (teacher-forced): 1e-5 max-abs
  * per step against the FP64 oracle: 1e-5 on the FP32 paths, 1e-4 where the workload states it
  * bit-identical where the same kernels see the same data (batched vs one world at a time)
"""
import os

import numpy as np
import pytest

import auto_gb300 as ag
from auto_gb300 import LeniaError, Sim, configs
from auto_gb300 import _lib
from oracle.oracle import fp64_convolve, fp64_step

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

FP32_PATHS = ["fp32", "radix2"]


@pytest.fixture(scope="module", autouse=True)
def built():
    from auto_gb300 import native
    native.build()
    _lib.load()


@pytest.fixture(scope="module")
def golden():
    return np.load(os.path.join(GOLDEN, "lenia_128x64.npz")), np.load(os.path.join(GOLDEN, "orbium.npy"))


@pytest.mark.parametrize("path", FP32_PATHS)
def test_reference_known_answer(golden, path):
    """tests/automata.rs:300-362 restated: 128x64, Orbium seed, one step vs f64 direct convolution."""
    g, _ = golden
    with Sim(ag.lenia(128, 64), path=path) as sim:
        sim.write_state(0, g["state0"])
        sim.step(1)
        got = sim.read_state(0)[0]
    worst = np.abs(got - g["want_direct"]).max()
    assert worst < float(g["tolerance"])
    assert worst < 1e-5, worst


@pytest.mark.parametrize("path", FP32_PATHS)
def test_orbium_tiles_seeded_on_device(golden, path):
    g, orb = golden
    pat = orb.astype(np.float32) / np.float32(255.0)
    with Sim(ag.lenia(128, 64, pattern=pat), seed=int(g["seed"]), path=path) as sim:
        assert np.array_equal(sim.read_state(0)[0], g["state0"])


@pytest.mark.parametrize("w,h", [(256, 128), (192, 192), (768, 384), (4096, 64), (96, 3072), (8192, 32), (6144, 64)])
def test_row_spectrum_matches_numpy(w, h):
    """The engine keeps, between steps, the half-spectrum along x of every row (the column
    transform happens inside the column pass)."""
    rng = np.random.default_rng(w + h)
    s = rng.random((h, w), dtype=np.float32)
    world = ag.World(w, h, [ag.Kernel(radius=10.0)])
    with Sim(world) as sim:
        sim.write_state(0, s)
        got = sim.spectrum(0)
    want = np.fft.rfft(s.astype(np.float64), axis=1)
    assert np.abs(got - want).max() / np.abs(want).max() < 2e-7


@pytest.mark.parametrize("w,h,R,beta", [(256, 256, 13.0, [1.0]), (128, 64, 13.0, [1.0]), (384, 192, 40.0, [1.0]),
                                         (1024, 1024, 52.0, [1.0, 0.5, 0.25]), (48, 96, 9.0, [0.3, 1.0])])
def test_u_field_matches_fp64(w, h, R, beta):
    rng = np.random.default_rng(int(R))
    s = rng.random((h, w), dtype=np.float32)
    world = ag.World(w, h, [ag.Kernel(radius=R, beta=beta)])
    with Sim(world) as sim:
        sim.write_state(0, s)
        u = sim.u_field(0, 0)
    want = fp64_convolve(world, s[None])[0]
    assert np.abs(u - want).max() < 2e-6


@pytest.mark.parametrize("path", FP32_PATHS)
def test_config1_teacher_forced_vs_reference_step(ref, path):
    """256x256, R=13: per step, the engine's step from state s_t vs the f32 restatement of the
    reference's step from the same s_t, and vs FP64."""
    world = configs.single_256()
    spectra = ref.spectra(world)
    worst_ref = worst_64 = 0.0
    with Sim(world, seed=configs.SEED_256, path=path) as sim:
        s = sim.read_state(0)[0]
        assert np.array_equal(s, ref.seed_patches(256, 256, configs.SEED_256, [(96, 96, 64, 64)]))
        for t in range(60):
            sim.step(1)
            got = sim.read_state(0)[0]
            want = ref.step(world, s, spectra=spectra, threads=1)
            worst_ref = max(worst_ref, float(np.abs(got - want).max()))
            if t % 10 == 0:
                worst_64 = max(worst_64, float(np.abs(got - fp64_step(world, s)[0]).max()))
            s = got
    assert worst_ref < 1e-5, worst_ref
    assert worst_64 < 1e-5, worst_64


def test_config2_4096_vs_fp64():
    world = configs.single_4096()
    with Sim(world, seed=configs.SEED_4096) as sim:
        s = sim.read_state(0)
        worst = 0.0
        for t in range(2):
            sim.step(1)
            got = sim.read_state(0)
            worst = max(worst, float(np.abs(got - fp64_step(world, s)).max()))
            s = got
    assert worst < 1e-5, worst


def test_full_size_translation_equivariance():
    """Size-independent property at 4096^2: stepping a torus-shifted state equals shifting the stepped state."""
    world = configs.single_4096()
    with Sim(world, seed=configs.SEED_4096) as sim:
        sim.step(3)
        s = sim.read_state(0)
        sim.step(2)
        a = sim.read_state(0)
        sim.write_state(0, np.roll(s, (123, 457), axis=(1, 2)))
        sim.step(2)
        b = sim.read_state(0)
    assert np.abs(np.roll(a, (123, 457), axis=(1, 2)) - b).max() < 1e-5


def test_full_size_uniform_field():
    world = configs.single_4096()
    with Sim(world) as sim:
        sim.write_state(0, np.full((1, 4096, 4096), 0.3, np.float32))
        sim.step(1)
        got = sim.read_state(0)
    k = world.kernels[0]
    d = (0.3 - k.mu) / k.sigma
    want = np.clip(0.3 + world.dt * (2 * np.exp(-0.5 * d * d) - 1), 0, 1)
    assert np.abs(got - want).max() < 2e-6


def test_batched_worlds_equal_one_at_a_time():
    worlds = configs.batched(48)
    with Sim(worlds, seed=0) as sim:
        for i, w in enumerate(worlds):
            sim.seed_patches(i, i, w.seed.patches)
        start = [sim.read_state(i) for i in range(len(worlds))]
        sim.step(4)
        batched = [sim.read_state(i) for i in range(len(worlds))]
    for i in (0, 1, 2, 5, 11, 23, 47):
        with Sim(worlds[i], seed=i) as one:
            one.write_state(0, start[i])
            one.step(4)
            assert np.array_equal(one.read_state(0), batched[i]), i


def test_all_world_state_calls_match_per_world_calls():
    # lenia_write_states / lenia_read_states (one copy for every world) against the per-world calls,
    # and the deferred spectrum refresh: partial rewrites, whole-context rewrites, then steps
    worlds = configs.batched(40)
    rng = np.random.default_rng(5)
    states = [rng.random((w.channels, w.height, w.width), dtype=np.float32) for w in worlds]
    flat = np.concatenate([s.ravel() for s in states])
    with Sim(worlds, seed=0) as a, Sim(worlds, seed=0) as b:
        a.write_states(flat)
        for i, s in enumerate(states):
            b.write_state(i, s)
        assert np.array_equal(a.read_states(), flat)
        a.step(3)
        b.step(3)
        got = a.read_states()
        off = 0
        for i, w in enumerate(worlds):
            n = w.channels * w.height * w.width
            assert np.array_equal(got[off:off + n], b.read_state(i).ravel()), i
            off += n
        # rewrite a few worlds only (one launch per changed world), then step both again
        for i in (0, 7, 39):
            a.write_state(i, states[i])
            b.write_state(i, states[i])
        a.step(2)
        b.step(2)
        got = a.read_states()
        off = 0
        for i, w in enumerate(worlds):
            n = w.channels * w.height * w.width
            assert np.array_equal(got[off:off + n], b.read_state(i).ravel()), i
            off += n
        with pytest.raises(LeniaError):
            a.write_states(flat[:-1])
        with pytest.raises(LeniaError):
            a.read_states(np.empty(flat.size + 1, np.float32))


@pytest.mark.parametrize("w,h,nk", [(8192, 64, 1), (64, 8192, 1), (6144, 96, 1), (96, 6144, 1), (8192, 64, 2)])
def test_largest_sides_teacher_forced_vs_fp64(w, h, nk):
    # the largest sides (up to 8192, 1024-thread CTAs) along either axis, one step from a random state;
    # nk = 2: the general step at the largest width
    kernels = [ag.Kernel(radius=13.0, beta=[1.0, 0.5])] + [ag.Kernel(radius=9.0, mu=0.2, sigma=0.02, weight=0.5)] * (nk - 1)
    world = ag.World(w, h, kernels, dt=0.1)
    rng = np.random.default_rng(w * 7 + h)
    s = rng.random((1, h, w), dtype=np.float32)
    with Sim(world) as sim:
        sim.write_state(0, s)
        sim.step(1)
        got = sim.read_state(0)
    assert np.abs(got - fp64_step(world, s)).max() < 1e-4


SIDES = [32, 48, 64, 96, 128, 192, 256, 384, 512, 768, 1024, 1536, 2048, 3072, 4096, 6144, 8192]


@pytest.mark.parametrize("nk,tune", [(1, False), (2, False), (1, True), (2, True)])
def test_every_side_on_both_axes_teacher_forced_vs_fp64(nk, tune):
    """Every supported side as the width (the row pass at that length) and as the height (the
    column pass), the other side 32, all in one context, one step from a random state.  nk = 1
    runs the single-kernel builds, nk = 2 the general ones; with tune the autotuner first times
    both launch variants of every size class and keeps the faster."""
    kernels = [ag.Kernel(radius=5.0, beta=[1.0, 0.5])] + [ag.Kernel(radius=3.0, mu=0.2, sigma=0.03, weight=0.5)] * (nk - 1)
    worlds = [ag.World(n, 32, kernels, dt=0.1) for n in SIDES] + [ag.World(32, n, kernels, dt=0.1) for n in SIDES[1:]]
    rng = np.random.default_rng(17 + nk)
    states = [rng.random((1, w.height, w.width), dtype=np.float32) for w in worlds]
    with Sim(worlds) as sim:
        for i, s in enumerate(states):
            sim.write_state(i, s)
        if tune:
            sim.autotune()
            assert all(np.array_equal(sim.read_state(i), s) for i, s in enumerate(states))
        sim.step(1)
        for i, w in enumerate(worlds):
            err = float(np.abs(sim.read_state(i) - fp64_step(w, states[i])).max())
            assert err < 1e-4, (w.width, w.height, err)


def test_async_state_copies_match_blocking_ones():
    """lenia_write_states_async / lenia_read_states_async, with two downloads in flight and an
    upload between steps, give the same bits as the blocking calls in the same order."""
    worlds = configs.batched(24)
    rng = np.random.default_rng(8)
    flat = np.concatenate([rng.random(w.channels * w.height * w.width, dtype=np.float32) for w in worlds])
    flat2 = flat[::-1].copy()
    outs = [np.empty_like(flat) for _ in range(3)]
    with Sim(worlds, seed=0) as a, Sim(worlds, seed=0) as b:
        a.write_states_async(flat)
        a.step(2)
        a.read_states_async(outs[0])
        a.step(3)
        a.read_states_async(outs[1])
        a.write_states_async(flat2)
        a.step(1)
        a.read_states_async(outs[2])
        a.wait()
        b.write_states(flat)
        b.step(2)
        want = [b.read_states().copy()]
        b.step(3)
        want.append(b.read_states().copy())
        b.write_states(flat2)
        b.step(1)
        want.append(b.read_states().copy())
        for got, w in zip(outs, want):
            assert np.array_equal(got, w)
        with pytest.raises(LeniaError):
            a.read_states_async(np.empty(flat.size + 1, np.float32))
    with Sim(configs.single_256(), path="radix2") as r:
        with pytest.raises(LeniaError):
            r.write_states_async(np.zeros(256 * 256, np.float32))


@pytest.mark.parametrize("nk", [1, 2])
def test_every_launch_variant_on_every_side(nk):
    """Each pinned pair of launch variants (column: scalar at 64 and 128 registers, paired, scalar
    with the radix-16 plan; row: the two register caps) on every supported side along either axis,
    one step vs FP64."""
    kernels = [ag.Kernel(radius=5.0, beta=[1.0, 0.5])] + [ag.Kernel(radius=3.0, mu=0.2, sigma=0.03, weight=0.5)] * (nk - 1)
    worlds = [ag.World(n, 32, kernels, dt=0.1) for n in SIDES] + [ag.World(32, n, kernels, dt=0.1) for n in SIDES[1:]]
    rng = np.random.default_rng(29 + nk)
    states = [rng.random((1, w.height, w.width), dtype=np.float32) for w in worlds]
    want = [fp64_step(w, s) for w, s in zip(worlds, states)]
    with Sim(worlds) as sim:
        for col in (0, 1, 2, 3):
            for row in (0, 1):
                sim.set_variants(col, row)
                assert set(sim.variants().values()) == {(col, row)}
                for i, s in enumerate(states):
                    sim.write_state(i, s)
                sim.step(1)
                for i, w in enumerate(worlds):
                    err = float(np.abs(sim.read_state(i) - want[i]).max())
                    assert err < 1e-4, (col, row, w.width, w.height, err)
        with pytest.raises(LeniaError):
            sim.set_variants(4, 0)
        with pytest.raises(LeniaError):
            sim.set_variants(0, 2)


def test_batched_worlds_teacher_forced_vs_fp64():
    worlds = configs.batched(32)
    with Sim(worlds, seed=0) as sim:
        for i, w in enumerate(worlds):
            sim.seed_patches(i, i, w.seed.patches)
        sim.step(5)
        before = [sim.read_state(i) for i in range(len(worlds))]
        sim.step(1)
        for i, w in enumerate(worlds):
            got = sim.read_state(i)
            want = fp64_step(w, before[i])
            assert np.abs(got - want).max() < 1e-4, (i, w.width)


def test_multichannel_teacher_forced_vs_fp64():
    world = configs.multichannel()
    with Sim(world, seed=configs.SEED_MULTI) as sim:
        s = sim.read_state(0)
        worst = 0.0
        for t in range(3):
            sim.step(1)
            got = sim.read_state(0)
            worst = max(worst, float(np.abs(got - fp64_step(world, s)).max()))
            s = got
    assert worst < 1e-4, worst


def test_multichannel_u_fields():
    world = configs.multichannel()
    rng = np.random.default_rng(11)
    s = rng.random((3, 1024, 1024), dtype=np.float32)
    with Sim(world) as sim:
        sim.write_state(0, s)
        us = [sim.u_field(0, k) for k in range(9)]
    want = fp64_convolve(world, s)
    for k in range(9):
        assert np.abs(us[k] - want[k]).max() < 2e-6, k


@pytest.mark.parametrize("path", FP32_PATHS)
def test_smoothlife_and_mnca(ref, path):
    rng = np.random.default_rng(5)
    s = (rng.random((256, 256)) < 0.4).astype(np.float32)
    for world in (ag.smoothlife(256, 256, 21.0), ag.mnca(256, 256)):
        with Sim(world, path=path) as sim:
            sim.write_state(0, s)
            u = [sim.u_field(0, k) for k in range(2)]
            sim.step(1)
            got = sim.read_state(0)[0]
        want_u = fp64_convolve(world, s[None])
        for k in range(2):
            assert np.abs(u[k] - want_u[k]).max() < 2e-6
        want_ref = ref.step(world, s)
        mismatch = np.abs(got - want_ref) > 1e-4
        # MNCA's bands are discontinuous: a U within rounding of a band edge may land either side
        assert mismatch.mean() < 1e-3, (world.id, mismatch.mean())


def test_stats():
    world = configs.single_256()
    with Sim(world, seed=configs.SEED_256) as sim:
        st = sim.stats()[0]
        s = sim.read_state(0)[0].astype(np.float64)
    assert abs(st[0] - s.sum()) / s.sum() < 1e-5
    ang = 2 * np.pi * np.arange(256) / 256
    cx = (np.arctan2((s.sum(0) * np.sin(ang)).sum(), (s.sum(0) * np.cos(ang)).sum()) / (2 * np.pi) * 256) % 256
    assert abs(st[1] - cx) < 1e-2


def test_errors_are_reported_not_raised_as_crashes():
    with pytest.raises(LeniaError) as e:
        Sim(ag.World(100, 100, [ag.Kernel()]))
    assert e.value.code == _lib.ESIZE
    with pytest.raises(LeniaError) as e:  # sides above 8192 are not built
        Sim(ag.World(16384, 64, [ag.Kernel()]))
    assert e.value.code == _lib.ESIZE
    with pytest.raises(LeniaError) as e:
        Sim(ag.World(64, 64, [ag.Kernel(radius=40.0)]))
    assert "smaller than its kernel" in str(e.value)
    with pytest.raises(LeniaError):
        Sim(ag.World(96, 64, [ag.Kernel()]), path="radix2")
    with Sim(ag.lenia(64, 64)) as sim:
        with pytest.raises(LeniaError):
            sim.write_state(0, np.zeros((1, 32, 32), np.float32))
        with pytest.raises(KeyError):
            sim.read_field("spec")


def test_graph_replay_matches_single_steps():
    """64-step graph replays give the same bits as 64 single-step replays."""
    world = configs.single_256()
    with Sim(world, seed=configs.SEED_256) as a, Sim(world, seed=configs.SEED_256) as b:
        a.step(64)
        for _ in range(64):
            b.step(1)
        assert np.array_equal(a.read_state(0), b.read_state(0))
        assert a.tick == b.tick == 64


def test_autotune_keeps_results():
    world = configs.single_256()
    with Sim(world, seed=configs.SEED_256) as a, Sim(world, seed=configs.SEED_256) as b:
        a.autotune()
        a.step(10)
        b.step(10)
        assert np.abs(a.read_state(0) - b.read_state(0)).max() < 1e-5


@pytest.mark.parametrize("kind,path", [(_lib.SEED_SL_DISCS, "fp32"), (_lib.SEED_MNCA_BLOCKS, "fp32"),
                                       (_lib.SEED_MNCA_BLOCKS, "radix2")])
def test_rule_seeds_on_device(ref, kind, path):
    world = ag.smoothlife(256, 256) if kind == _lib.SEED_SL_DISCS else ag.mnca(256, 256)
    with Sim(world, seed=7, path=path) as sim:
        got = sim.read_state(0)[0]
    want = ref.seed_sl_discs(256, 256, 7) if kind == _lib.SEED_SL_DISCS else ref.seed_mnca_blocks(256, 256, 7)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("palette,samples,scale,origin", [(0, 2, 1.0, (0.0, 0.0)), (1, 3, 2.5, (-10.0, 5.0)),
                                                          (2, 1, 0.5, (30.0, 40.0))])
def test_headless_view_matches_oracle(ref, palette, samples, scale, origin):
    rng = np.random.default_rng(palette)
    s = rng.random((192, 256), dtype=np.float32)
    with Sim(ag.World(256, 192, [ag.Kernel(radius=10.0)])) as sim:
        sim.write_state(0, s)
        img = sim.render(0, 200, 150, origin=origin, scale=scale, samples=samples, palette=palette)
    want = ref.render(s, 200, 150, origin=origin, scale=scale, samples=samples, palette=palette)
    diff = np.abs(img.astype(int) - want.astype(int))
    assert diff.max() <= 1 and (diff > 0).mean() < 1e-3


def test_chunked_classes_give_the_same_bits():
    """Splitting size classes into L2-sized runs of worlds only regroups the launches: every world's
    state after 6 steps is bit-identical with one run per class and with runs of a few worlds, and
    with the autotuner's shapes a step stays within 1e-5 of FP64; the shapes report the chunking."""
    worlds = configs.batched(64)
    outs = []
    for budget in (0, 8, 1):
        with Sim(worlds, seed=0) as sim:
            for i, w in enumerate(worlds):
                sim.seed_patches(i, i, w.seed.patches)
            sim.set_chunk_budget(budget)
            shapes = sim.shapes()
            if budget == 0:
                assert all(v["chunks"] == 1 for v in shapes.values())
            if budget == 1:  # every world of 512 and up is a chunk of its own
                assert all(v["chunks"] == v["worlds"] for (w, h), v in shapes.items() if w >= 512)
            sim.step(6)
            outs.append(sim.read_states().copy())
    assert np.array_equal(outs[0], outs[1]) and np.array_equal(outs[0], outs[2])
    # the autotuner's shapes: its launch variants may run other radix plans (radix 32, or the paired
    # radix-16 build), whose rounding differs and compounds over the steps; each step stays within
    # 1e-5 of FP64
    with Sim(worlds, seed=0) as sim:
        for i, w in enumerate(worlds):
            sim.seed_patches(i, i, w.seed.patches)
        sim.autotune()
        sim.step(5)
        before = [sim.read_state(i) for i in range(len(worlds))]
        sim.step(1)
        got = sim.read_states()
    assert np.abs(got - outs[0]).max() < 1e-4
    off, worst = 0, 0.0
    for w, s in zip(worlds, before):
        n = w.channels * w.height * w.width
        worst = max(worst, float(np.abs(got[off:off + n] - fp64_step(w, s).ravel()).max()))
        off += n
    assert worst < 1e-5, worst


def test_resident_step_matches_two_pass_and_fp64():
    """The cluster-resident step (one launch advances a class's worlds through every generation, one
    thread-block cluster per world with its half-spectrum in distributed shared memory) against the
    two launches per generation on the same worlds -- every side it serves, 128 to 512 -- after 1, 5
    and 64 more generations, and one step against FP64.  Its butterflies, packing and growth are the
    two-pass step's own device code, so the two agree to float rounding of the same operations."""
    worlds = [w for w in configs.batched(160) if w.width <= 512]
    assert {w.width for w in worlds} == {128, 192, 256, 384, 512}
    with Sim(worlds, seed=0) as a, Sim(worlds, seed=0) as b:
        for sim in (a, b):
            for i, w in enumerate(worlds):
                sim.seed_patches(i, i, w.seed.patches)
        a.set_resident(True)
        b.set_resident(False)
        assert all(v["resident"] == 1 for v in a.shapes().values())
        assert all(v["resident"] == 0 for v in b.shapes().values())
        worst = 0.0
        identical = True
        for steps in (1, 5, 64):
            a.step(steps)
            b.step(steps)
            sa, sb = a.read_states(), b.read_states()
            identical = identical and np.array_equal(sa, sb)
            worst = max(worst, float(np.abs(sa - sb).max()))
        a.wait()  # raises if a cluster sync gave up
        print("resident vs two-pass after 70 generations: max|diff| %.3e, bit-identical %s" % (worst, identical))
        assert worst < 1e-5, worst
        before = [a.read_state(i) for i in range(len(worlds))]
        a.step(1)
        for i, w in enumerate(worlds):
            err = float(np.abs(a.read_state(i) - fp64_step(w, before[i])).max())
            assert err < 1e-5, (i, w.width, err)
        # the engine's spectrum is current after a resident launch: a U-field read uses it
        u = a.u_field(0, 0)
        assert np.abs(u - fp64_convolve(worlds[0], a.read_state(0))[0]).max() < 2e-6


def test_resident_step_applies_only_where_it_can():
    """Classes the resident step does not serve (wider than 512, several kernels, the tensor-core
    paths) keep the two launches per generation whatever lenia_set_resident asks."""
    worlds = [configs.batched_world(i) for i in range(40)]
    big = [w for w in worlds if w.width > 512][:2]
    two = ag.World(256, 256, [ag.Kernel(radius=10.0), ag.Kernel(radius=6.0, mu=0.2, sigma=0.03, weight=0.5)])
    with Sim(big + [two], seed=0) as sim:
        sim.set_resident(True)
        assert all(v["resident"] == 0 for v in sim.shapes().values())
    with Sim([w for w in worlds if w.width == 256][:2], seed=0, path="bf16x3") as sim:
        sim.set_resident(True)
        assert all(v["resident"] == 0 for v in sim.shapes().values())


@pytest.mark.parametrize("path", ["fp32", "bf16x3"])
def test_two_branch_graph_gives_the_same_bits(path):
    """Running the small size classes on side graph branches beside the large ones (one side branch,
    or one each) only reorders independent launches: every state after 5 steps is bit-identical to
    one branch.  On the tensor-core path the side branches hold tensor-core classes too (256, 512)."""
    worlds = configs.batched(64)
    outs = []
    for split, each in ((0, False), (256 * 256, False), (512 * 512, False), (384 * 384, True)):
        with Sim(worlds, seed=0, path=path) as sim:
            for i, w in enumerate(worlds):
                sim.seed_patches(i, i, w.seed.patches)
            sim.set_branch_split(split, each)
            assert sim.branch_split == (split, each)
            sim.step(5)
            outs.append(sim.read_states().copy())
    for o in outs[1:]:
        assert np.array_equal(outs[0], o)


@pytest.mark.parametrize("path", ["fp32", "bf16x3"])
def test_chunk_lanes_give_the_same_bits(path):
    """A class's chunks on 2..4 concurrent graph lanes (each lane's chunks one after another) only
    reorder independent worlds' launches: every state after 9 steps is bit-identical to one chunk, and
    to the same chunks one after another.  The lanes sit on the main graph branch, with the small
    classes on a side branch."""
    ws = configs.batched(384)
    worlds = [w for w in ws if w.width in (256, 512, 768)][:30]
    outs = []
    for budget, lanes in ((0, 1), (8, 1), (8, 2), (8, 3), (8, 4)):
        with Sim(worlds, seed=0, path=path) as sim:
            for i, w in enumerate(worlds):
                sim.seed_patches(i, i, w.seed.patches)
            sim.set_branch_split(256 * 256, False)
            sim.set_chunk_budget(budget)
            sim.set_chunk_lanes(lanes)
            sh = sim.shapes()
            assert all(v["lanes"] == lanes for v in sh.values())
            if budget:
                assert sh[(768, 768)]["chunks"] > lanes
            sim.step(9)
            outs.append(sim.read_states().copy())
            if lanes == 4:
                with pytest.raises(LeniaError):
                    sim.set_chunk_lanes(0)
                with pytest.raises(LeniaError):
                    sim.set_chunk_lanes(5)
                # per class: the column and row launches each alone, and the class as the graph runs it
                prof = sim.profile_classes(2)
                assert set(prof) == set(sh) and all(c > 0 and r > 0 and g > 0 for c, r, g in prof.values())
    for o in outs[1:]:
        assert np.array_equal(outs[0], o)


def test_persistent_wait_timeout_reports_error_and_leaves_context_usable():
    """Failure detection of the persistent step, with no GPU fault: the test hook makes every
    dependency wait give up at once, so the launch's CTAs stop claiming items and return, and
    lenia_sync reports LENIA_ECUDA.  With the limit restored and the states rewritten (the failed step's
    spectra are invalid), the same context steps again in agreement with FP64."""
    ws = configs.batched(384)
    worlds = [w for w in ws if w.width == 256][:6]
    with Sim(worlds, seed=0) as sim:
        for i, w in enumerate(worlds):
            sim.seed_patches(i, i, w.seed.patches)
        sim.set_persistent(True)
        assert all(v["persistent"] >= 0 for v in sim.shapes().values())
        sim.set_persist_wait_limit(1)
        sim.step(4)
        with pytest.raises(LeniaError):
            sim.wait()
        with pytest.raises(LeniaError):
            sim.set_persist_wait_limit(-1)
        sim.set_persist_wait_limit(0)
        states = sim.read_states().copy()
        sim.write_states(states)
        sim.step(1)
        got = sim.read_states()
    off, worst = 0, 0.0
    for w in worlds:
        n = w.channels * w.height * w.width
        s = states[off:off + n].reshape(w.channels, w.height, w.width)
        worst = max(worst, float(np.abs(got[off:off + n] - fp64_step(w, s).ravel()).max()))
        off += n
    assert worst < 1e-5, worst


@pytest.mark.parametrize("variant", [0, 1])
def test_persistent_step_matches_two_pass_bit_for_bit(variant):
    """The persistent step (one launch a class and step call, items claimed in order with per-world
    dependencies), in both launch variants, runs the two-pass step's item code on the same inputs:
    bit-identical states after 70 generations on batched worlds of every side it serves, no wait given
    up, and within 1e-5 of FP64 at the last step."""
    from oracle.oracle import fp64_step
    ws = configs.batched(384)
    worlds = []
    for side in (128, 192, 256, 384, 512, 768, 1024):
        worlds += [w for w in ws if w.width == side][:3]
    out = []
    for on in (False, True):
        with Sim(worlds, seed=0) as sim:
            for i, w in enumerate(worlds):
                sim.seed_patches(i, i, w.seed.patches)
            sim.set_persistent(on, variant)
            assert all(v["persistent"] == (variant if on else -1) for v in sim.shapes().values())
            sim.step(69)
            before = [sim.read_state(i) for i in range(len(worlds))]
            sim.step(1)
            sim.wait()
            out.append(sim.read_states().copy())
    assert np.array_equal(out[0], out[1])
    off = 0
    for i, w in enumerate(worlds):
        n = w.width * w.height
        err = float(np.abs(out[1][off:off + n].reshape(1, w.height, w.width) - fp64_step(w, before[i])).max())
        assert err < 1e-5, (i, w.width, err)
        off += n


def test_persistent_step_single_4096():
    """The persistent step on one 4096 x 4096 world (configuration 2): bit-identical after 6 steps to
    the two-pass step in its scalar column build (the persistent step's column items are the scalar
    build's; the two-pass default at 4096, the paired f32x2 build, rounds differently), and within
    1e-5 of FP64 at the last step."""
    world = configs.single_4096()
    out = []
    for on in (False, True):
        with Sim(world, seed=configs.SEED_4096) as sim:
            if on:
                sim.set_persistent(True)
            else:
                sim.set_variants(0, -1)
            sim.step(5)
            before = sim.read_state(0).copy()
            sim.step(1)
            out.append(sim.read_state(0).copy())
    assert np.array_equal(out[0], out[1])
    err = float(np.abs(out[1] - fp64_step(world, before)).max())
    assert err < 1e-5, err
