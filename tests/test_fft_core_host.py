"""The shared-memory FFT templates (auto_gb300/csrc/fft_core.cuh), built for the host with g++
and run stage by stage as the GPU does, against numpy's FFT."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT

SIZES = [16, 32, 48, 64, 96, 128, 192, 256, 384, 512, 768, 1024, 1536, 2048, 3072, 4096, 8192]


@pytest.fixture(scope="module")
def fft_host(tmp_path_factory):
    if not shutil.which("g++"):
        pytest.skip("g++ not available")
    out = str(tmp_path_factory.mktemp("fft") / "fft_host.so")
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-shared", "-fPIC",
                           os.path.join(ROOT, "tests", "cpp", "fft_core_host.cpp"), "-o", out])
    return ctypes.CDLL(out)


@pytest.mark.parametrize("n", SIZES)
@pytest.mark.parametrize("inverse", [0, 1])
def test_stockham_plan_matches_numpy(fft_host, n, inverse):
    rng = np.random.default_rng(n + inverse)
    x = (rng.random(n) + 1j * rng.random(n)).astype(np.complex64)
    out = np.zeros(n, np.complex64)
    assert fft_host.fft_host(n, inverse, x.ctypes.data_as(ctypes.c_void_p), out.ctypes.data_as(ctypes.c_void_p)) == 0
    x64 = x.astype(np.complex128)
    want = np.fft.ifft(x64) * n if inverse else np.fft.fft(x64)
    assert np.abs(out - want).max() / np.abs(want).max() < 2e-7


@pytest.mark.parametrize("n", SIZES)
@pytest.mark.parametrize("inverse", [0, 1])
def test_radix32_plans_match_numpy(fft_host, n, inverse):
    """The plans a pass gets when it allows radix 32 (radix 32 where that saves a stage: 1024,
    3072, 8192; the radix-16 plan elsewhere), with their twiddle powers up to w^31 and the radix-32
    stores, against numpy."""
    rng = np.random.default_rng(2000 + n + inverse)
    x = (rng.random(n) + 1j * rng.random(n)).astype(np.complex64)
    out = np.zeros(n, np.complex64)
    assert fft_host.fft_host_r32(n, inverse, x.ctypes.data_as(ctypes.c_void_p), out.ctypes.data_as(ctypes.c_void_p)) == 0
    x64 = x.astype(np.complex128)
    want = np.fft.ifft(x64) * n if inverse else np.fft.fft(x64)
    assert np.abs(out - want).max() / np.abs(want).max() < 2e-7


@pytest.mark.parametrize("n", SIZES)
@pytest.mark.parametrize("inverse", [0, 1])
def test_paired_sequences_match_numpy(fft_host, n, inverse):
    """Two sequences through the same stages as cpair elements (re and im planes of both in one
    16-byte element, twiddles held twice): each must come out as its own FFT."""
    rng = np.random.default_rng(1000 + n + inverse)
    a = (rng.random(n) + 1j * rng.random(n)).astype(np.complex64)
    b = (rng.random(n) - 1j * rng.random(n)).astype(np.complex64)
    oa, ob = np.zeros(n, np.complex64), np.zeros(n, np.complex64)
    ptr = lambda x: x.ctypes.data_as(ctypes.c_void_p)
    assert fft_host.fft_host_pair(n, inverse, ptr(a), ptr(b), ptr(oa), ptr(ob)) == 0
    for x, out in ((a, oa), (b, ob)):
        x64 = x.astype(np.complex128)
        want = np.fft.ifft(x64) * n if inverse else np.fft.fft(x64)
        assert np.abs(out - want).max() / np.abs(want).max() < 2e-7


@pytest.mark.parametrize("maxr", [32, 16, 8])
def test_radix_plans(fft_host, maxr):
    """Every plan multiplies out to its length, uses only built radices within the cap, and starts
    and ends with the same radix (the chained transforms rely on it)."""
    for n in SIZES:
        out = (ctypes.c_int * 14)()
        k = fft_host.plan_host(n, maxr, out)
        r = list(out[:k])
        assert int(np.prod(r)) == n, (n, r)
        assert all(x in (2, 3, 4, 8, 16, 32) and x <= maxr for x in r), (n, r)
        if n >= 16:
            assert k >= 2 and r[0] == r[-1], (n, r)
    out = (ctypes.c_int * 14)()
    k = fft_host.plan_host(4096, 16, out)
    assert list(out[:k]) == [16, 16, 16]
    k = fft_host.plan_host(3072, 16, out)
    assert list(out[:k]) == [16, 3, 4, 16]
    # radix 32 only where it saves a stage
    for n, want in ((1024, [32, 32]), (3072, [32, 3, 32]), (8192, [32, 8, 32]), (4096, [16, 16, 16]),
                    (2048, [16, 8, 16]), (512, [16, 2, 16])):
        k = fft_host.plan_host(n, 32, out)
        assert list(out[:k]) == want, (n, list(out[:k]))
