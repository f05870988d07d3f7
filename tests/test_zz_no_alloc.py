"""lenia_step_noalloc: stepping a world without any device allocation by the library.

Callers such as an application whose device memory all belongs to its own pool allocator, or a
frame loop that must not stall on an allocation, own the state and the kernel spectrum and pass
device pointers; the library's own scratch is a fixed array inside the loaded module.  This test
calls the entry point through the C ABI twice in a row on the same state and checks each result
against the ordinary context entry points (lenia_create / lenia_step) on the same world, within
the per-step tolerance of the parity tests (1e-5 max-abs).  The file is named so that pytest
collects it last; it also passes on its own in a fresh process.
"""
import ctypes

import numpy as np
import pytest

import auto_gb300 as ag
from auto_gb300 import Sim, _lib

pytestmark = pytest.mark.gpu


# 1024 x 1024 fills the half-spectrum region exactly; 4096 x 256 fills the column-item region and
# 256 x 4096 the row-item region.
@pytest.mark.parametrize("w,h", [(512, 256), (1024, 1024), (4096, 256), (256, 4096)])
def test_noalloc_matches_context_step_on_two_calls(w, h):
    torch = pytest.importorskip("torch")
    from auto_gb300 import native
    native.build()
    L = _lib.load()
    k = ag.Kernel(radius=20.0, beta=[1.0, 0.5], mu=0.2, sigma=0.03)
    world = ag.World(w, h, [k], dt=0.1)
    rng = np.random.default_rng(3 + w + h)
    s0 = np.zeros((h, w), np.float32)
    s0[h // 4:3 * h // 4, w // 4:3 * w // 4] = rng.random((h // 2, w // 2), dtype=np.float32)

    kd = world.to_desc().kernels[0]
    khat = np.zeros((w // 2 + 1) * (h // 2 + 1), np.float32)
    assert L.lenia_kernel_spectrum(ctypes.byref(kd), w, h, _lib.fptr(khat), khat.size) == 0
    # the caller's own device buffers
    d_state = torch.from_numpy(s0.copy()).cuda()
    d_khat = torch.from_numpy(khat).cuda()
    torch.cuda.synchronize()

    with Sim(world) as sim:
        sim.write_state(0, s0)
        for steps in (3, 2):
            rc = L.lenia_step_noalloc(ctypes.c_void_p(d_state.data_ptr()), w, h, ctypes.c_void_p(d_khat.data_ptr()),
                                      k.mu, k.sigma, world.dt, steps, None)
            assert rc == 0, L.lenia_last_error(None)
            torch.cuda.synchronize()
            sim.step(steps)
            want = sim.read_state(0)[0]
            got = d_state.cpu().numpy()
            assert np.abs(got - want).max() < 1e-5


def test_noalloc_rejects_worlds_over_its_limit():
    from auto_gb300 import native
    native.build()
    L = _lib.load()
    one = ctypes.c_void_p(16)  # never dereferenced: the size check comes first
    rc = L.lenia_step_noalloc(one, 2048, 1024, one, 0.15, 0.015, 0.1, 1, None)
    assert rc == _lib.ESIZE
    assert b"at most 1048576" in L.lenia_last_error(None)
