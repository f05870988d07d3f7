"""The C ABI library on a machine without a GPU: it loads, exports every declared entry point,
and its host-only parts (kernel spectra, validation) agree with the oracle.  No kernel launches."""
import ctypes
import os
import re

import numpy as np
import pytest

import auto_gb300 as ag
from auto_gb300 import _lib
from oracle.oracle import fp64_khat

from conftest import ROOT


def declared():
    src = open(os.path.join(ROOT, "include", "lenia_gb300.h")).read()
    return sorted(set(re.findall(r"LENIA_API\s+[\w\s\*]*?\b(lenia_\w+)\s*\(", src)))


def test_every_declared_symbol_is_exported(engine_lib):
    names = declared()
    assert len(names) >= 20
    for n in names:
        assert hasattr(engine_lib, n), n
    assert sorted(_lib.EXPORTS) == names


def kernel_desc(shape=ag.SHAPE_LENIA, radius=13.0, beta=(1.0,), lo=0.0, hi=0.0):
    k = _lib.LeniaKernel()
    k.shape, k.radius, k.nshells = shape, radius, len(beta)
    for i, b in enumerate(beta):
        k.beta[i] = b
    k.ring_lo, k.ring_hi, k.sigma, k.weight = lo, hi, 1.0, 1.0
    return k


@pytest.mark.parametrize("w,h,kw", [
    (256, 256, dict(radius=13.0)),
    (128, 64, dict(radius=13.0)),
    (192, 384, dict(radius=40.0)),
    (768, 768, dict(radius=25.0, beta=(1.0, 0.5, 0.25))),
    (256, 256, dict(shape=ag.SHAPE_SL_INNER, radius=21.0)),
    (256, 256, dict(shape=ag.SHAPE_SL_OUTER, radius=21.0)),
    (96, 96, dict(shape=ag.SHAPE_RING, lo=12.0, hi=18.0)),
])
def test_kernel_spectrum_matches_fp64_oracle(engine_lib, w, h, kw):
    k = kernel_desc(**kw)
    out = np.zeros((w // 2 + 1) * (h // 2 + 1), np.float32)
    rc = engine_lib.lenia_kernel_spectrum(ctypes.byref(k), w, h, _lib.fptr(out), out.size)
    assert rc == 0, engine_lib.lenia_last_error(None)
    got = out.reshape(w // 2 + 1, h // 2 + 1).T.astype(np.float64) * (w * h)
    spec = ag.Kernel(shape=k.shape, radius=k.radius, beta=list(kw.get("beta", (1.0,))), lo=k.ring_lo, hi=k.ring_hi)
    want = fp64_khat(w, h, spec)[: h // 2 + 1, :]
    assert np.abs(got - want).max() < 1e-6


def test_kernel_spectrum_rejects_bad_sizes(engine_lib):
    k = kernel_desc(radius=40.0)
    out = np.zeros(65 * 65, np.float32)
    assert engine_lib.lenia_kernel_spectrum(ctypes.byref(k), 64, 64, _lib.fptr(out), out.size) == _lib.ESIZE
    assert b"smaller than its kernel" in engine_lib.lenia_last_error(None)
    k = kernel_desc(radius=13.0)
    assert engine_lib.lenia_kernel_spectrum(ctypes.byref(k), 100, 64, _lib.fptr(out), out.size) == _lib.ESIZE
    assert engine_lib.lenia_kernel_spectrum(ctypes.byref(k), 64, 64, _lib.fptr(out), 7) == _lib.EINVAL


def test_registry_mirrors_reference_entries():
    assert [e.id for e in ag.ALL] == ["lenia", "smoothlife", "mnca"]
    w = ag.build("lenia", 100, 60)
    assert (w.width, w.height) == (128, 64)
    assert w.kernels[0].radius == 13.0 and w.kernels[0].mu == 0.15 and w.dt == 0.1
    assert ag.build("mnca.12,18,3,8", 256, 256).kernels[1].hi == 8.0
    assert ag.build("nope", 64, 64) is None
    sl = ag.build("smoothlife", 512, 512)
    assert sl.rule == ag.RULE_SMOOTHLIFE and len(sl.kernels) == 2


def test_configs_are_deterministic():
    a = ag.configs.single_4096_patches()
    assert a == ag.configs.single_4096_patches()
    assert all(0 <= x < 3840 and 0 <= y < 3840 for x, y, _, _ in a)
    ws = ag.configs.batched(384)
    assert len(ws) == 384 and {w.width for w in ws} == set(ag.configs.BATCH_SIDES)
    for w in ws:
        k = w.kernels[0]
        assert 8 <= k.radius <= 40 and 0.10 <= k.mu <= 0.35 and 0.01 <= k.sigma <= 0.06 and 0.05 <= w.dt <= 0.2
        assert 2 * k.radius < w.width
    m = ag.configs.multichannel()
    for d in range(3):
        assert abs(sum(k.weight for k in m.kernels if k.dst == d) - 1.0) < 1e-6


def test_rust_crate_binds_only_declared_entry_points():
    """crates/auto-cuda (not compiled here: no Rust toolchain) binds the C ABI by name: every
    function in its extern block is one the header declares, with the same number of arguments."""
    src = open(os.path.join(ROOT, "crates", "auto-cuda", "src", "lib.rs")).read()
    block = src[src.index('unsafe extern "C" {'):]
    block = block[:block.index("\n}\n")]
    rust = dict(re.findall(r"fn (lenia_\w+)\(([^)]*)\)", block.replace("\n", " ")))
    hdr = open(os.path.join(ROOT, "include", "lenia_gb300.h")).read().replace("\n", " ")
    c = dict(re.findall(r"LENIA_API\s+[\w\s\*]*?\b(lenia_\w+)\s*\(([^)]*)\)", hdr))
    assert len(rust) >= 15
    for name, args in rust.items():
        assert name in c, name
        assert len([a for a in args.split(",") if a.strip()]) == len([a for a in c[name].split(",") if a.strip()]), name
