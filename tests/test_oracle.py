"""The oracle against the reference's own known-answer test and golden vectors (CPU only).

The reference pins its Lenia step with one test (crates/auto-core/tests/automata.rs:300-362):
128x64, R=13, the first seed in 1..64 that places an Orbium, one step, compared with an f64
direct torus convolution, max|delta| < 2e-3.  tests/golden/gen_golden.py restated that test's
inputs and expected output from the reference sources; here the oracle must reproduce them.
"""
import os

import numpy as np
import pytest

from oracle.oracle import (RULE_LENIA, RULE_MNCA, RULE_SMOOTHLIFE, SHAPE_LENIA, SHAPE_RING, SHAPE_SL_INNER,
                           SHAPE_SL_OUTER, fp64_khat, fp64_kernel_spatial, fp64_step)
from types import SimpleNamespace as NS

from conftest import GOLDEN


def lenia_world(w, h, R=13.0, beta=(1.0,), mu=0.15, sigma=0.015, dt=0.1):
    k = NS(shape=SHAPE_LENIA, radius=R, beta=list(beta), lo=0.0, hi=0.0, src=0, dst=0, mu=mu, sigma=sigma, weight=1.0)
    return NS(width=w, height=h, channels=1, kernels=[k], dt=dt, rule=RULE_LENIA)


@pytest.fixture(scope="module")
def golden():
    g = np.load(os.path.join(GOLDEN, "lenia_128x64.npz"))
    orb = np.load(os.path.join(GOLDEN, "orbium.npy"))
    return g, orb


def test_pcg_vectors(ref):
    v = np.load(os.path.join(GOLDEN, "pcg_vectors.npz"))
    for t, r, u in zip(v["triples"], v["rand3"], v["unit_f"]):
        assert ref.rand3(int(t[0]), int(t[1]), int(t[2])) == int(r)
        assert np.float32(ref.unit_f(int(r))) == u


def test_orbium_seed_matches_golden(ref, golden):
    g, orb = golden
    s = ref.seed_tiles(128, 64, int(g["seed"]), orb.astype(np.float32) / np.float32(255.0))
    assert np.array_equal(s, g["state0"])
    assert (s > 0).any()


def test_direct_convolution_matches_golden(ref, golden):
    g, _ = golden
    d = ref.direct_lenia_step(g["state0"])
    assert np.abs(d - g["want_direct"]).max() <= 1e-6


def test_f32_restatement_matches_reference_test(ref, golden):
    """tests/automata.rs:361 asserts worst < 0.002; the restatement is far inside it."""
    g, _ = golden
    got = ref.step(lenia_world(128, 64), g["state0"])
    worst = np.abs(got - g["want_direct"]).max()
    assert worst < float(g["tolerance"])
    assert worst < 1e-5


def test_fp64_oracle_matches_reference_test(golden):
    g, _ = golden
    got = fp64_step(lenia_world(128, 64), g["state0"])[0]
    assert np.abs(got - g["want_direct"]).max() < 1e-6


def test_kernel_sum_and_dc():
    w = lenia_world(256, 256, R=13.0)
    k = w.kernels[0]
    sp = fp64_kernel_spatial(256, 256, k)
    assert abs(sp.sum() - 1.0) < 1e-12
    kh = fp64_khat(256, 256, k)
    assert abs(kh[0, 0] - 1.0) < 1e-12
    # even kernel -> real spectrum
    full = np.fft.fft2(sp)
    assert np.abs(full.imag).max() < 1e-12


def test_uniform_field_is_a_fixed_point_of_the_convolution(ref):
    w = lenia_world(64, 64)
    s = np.full((64, 64), 0.2, np.float32)
    out, conv = ref.step(w, s, return_conv=True)
    assert np.abs(conv[0] - 0.2).max() < 1e-6
    d = (0.2 - 0.15) / 0.015
    want = np.clip(0.2 + 0.1 * (2 * np.exp(-0.5 * d * d) - 1), 0, 1)
    assert np.abs(out - want).max() < 1e-6


@pytest.mark.parametrize("size", [(64, 64), (128, 64), (256, 128)])
def test_f32_restatement_vs_fp64_random(ref, size):
    w, h = size
    rng = np.random.default_rng(7)
    s = np.zeros((h, w), np.float32)
    s[h // 4: 3 * h // 4, w // 4: 3 * w // 4] = rng.random((h // 2, w // 2), dtype=np.float32)
    world = lenia_world(w, h)
    a = ref.step(world, s)
    b = fp64_step(world, s)[0]
    assert np.abs(a - b).max() < 1e-5


def test_multishell_kernel_restatements_agree(ref):
    """The C and numpy shape functions agree on Chan's multi-shell kernel."""
    w = lenia_world(256, 256, R=52.0 / 4, beta=(1.0, 0.5, 0.25), mu=0.26, sigma=0.036, dt=0.05)
    a = ref.kernel_spatial(256, 256, w.kernels[0]).astype(np.float64)
    b = fp64_kernel_spatial(256, 256, w.kernels[0])
    assert np.abs(a - b).max() < 1e-7


def test_smoothlife_and_mnca_restatements_agree(ref):
    rng = np.random.default_rng(3)
    s = (rng.random((128, 128)) < 0.3).astype(np.float32)
    sl = NS(width=128, height=128, channels=1, dt=0.1, rule=RULE_SMOOTHLIFE,
            kernels=[NS(shape=SHAPE_SL_INNER, radius=9.0, beta=[1.0], lo=0, hi=0, src=0, dst=0, mu=0, sigma=1, weight=1),
                     NS(shape=SHAPE_SL_OUTER, radius=9.0, beta=[1.0], lo=0, hi=0, src=0, dst=0, mu=0, sigma=1, weight=1)])
    a, ca = ref.step(sl, s, return_conv=True)
    from oracle.oracle import fp64_convolve
    cb = fp64_convolve(sl, s)
    assert np.abs(ca - cb).max() < 1e-5
    mn = NS(width=128, height=128, channels=1, dt=0.1, rule=RULE_MNCA,
            kernels=[NS(shape=SHAPE_RING, radius=0, beta=[1.0], lo=12.0, hi=18.0, src=0, dst=0, mu=0, sigma=1, weight=1),
                     NS(shape=SHAPE_RING, radius=0, beta=[1.0], lo=3.0, hi=8.0, src=0, dst=0, mu=0, sigma=1, weight=1)])
    _, cm = ref.step(mn, s, return_conv=True)
    assert np.abs(cm - fp64_convolve(mn, s)).max() < 1e-5


def test_reference_rejects_non_power_of_two(ref):
    with pytest.raises(ValueError):
        ref.step(lenia_world(96, 64), np.zeros((64, 96), np.float32))
