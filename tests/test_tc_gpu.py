"""Tensor-core (tcgen05) path on a GB300: the GEMM self-test through the operand layouts and
descriptors the column pass uses, then the TF32 / BF16x3 step against the FP64 oracle.

Tolerances: the self-test GEMM against float64 (TF32 1e-2 relative, BF16x3 2e-4 relative, as the
operand roundings allow); the BF16x3 step per step against FP64 within 1e-4 max-abs (the target
precision of the tensor-core path); TF32 is reported, with a looser bound of 5e-3."""
import numpy as np
import pytest

import auto_gb300 as ag
from auto_gb300 import Sim, configs
from auto_gb300 import _lib
from oracle.oracle import fp64_convolve, fp64_step

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    from auto_gb300 import native
    native.build()
    _lib.load()


@pytest.mark.parametrize("path,tol", [(_lib.PATH_BF16X3, 2e-4), (_lib.PATH_TF32, 1e-2)])
@pytest.mark.parametrize("n,k", [(128, 128), (64, 64), (32, 32), (256, 128)])
def test_gemm_selftest(path, tol, n, k):
    rng = np.random.default_rng(n * k + path)
    a = rng.standard_normal((128, k)).astype(np.float32)
    b = rng.standard_normal((n, k)).astype(np.float32)
    d = np.zeros((128, n), np.float32)
    rc = _lib.load().lenia_tc_selftest(path, n, k, _lib.fptr(a), _lib.fptr(b), _lib.fptr(d))
    assert rc == 0, _lib.load().lenia_last_error(None)
    want = a.astype(np.float64) @ b.astype(np.float64).T
    err = np.abs(d - want).max() / np.abs(want).max()
    assert err < tol, err


@pytest.mark.parametrize("n,k", [(64, 64), (128, 64), (32, 32), (256, 16)])
def test_gemm_selftest_mn_major_a(n, k):
    """The MN-major A operand of the transposing hand-overs (8 consecutive rows of one k in 16 bytes;
    MN-adjacent core matrices 128 bytes apart, K-adjacent groups of 8 K M/8 core matrices apart),
    BF16x3, against float64."""
    rng = np.random.default_rng(n * k + 11)
    a = rng.standard_normal((128, k)).astype(np.float32)
    b = rng.standard_normal((n, k)).astype(np.float32)
    d = np.zeros((128, n), np.float32)
    rc = _lib.load().lenia_tc_selftest(_lib.PATH_BF16X3 | _lib.SELFTEST_A_MN, n, k, _lib.fptr(a), _lib.fptr(b),
                                       _lib.fptr(d))
    assert rc == 0, _lib.load().lenia_last_error(None)
    want = a.astype(np.float64) @ b.astype(np.float64).T
    err = np.abs(d - want).max() / np.abs(want).max()
    assert err < 2e-4, err


@pytest.mark.parametrize("path", ["bf16x3", "tf32"])
@pytest.mark.parametrize("side", [256, 512, 1024, 2048, 4096])
def test_tc_u_field_vs_fp64(path, side):
    rng = np.random.default_rng(side)
    s = rng.random((side, side), dtype=np.float32)
    world = ag.World(side, side, [ag.Kernel(radius=min(52.0, side / 4), beta=[1.0, 0.5, 0.25])])
    with Sim(world, path=path) as sim:
        sim.write_state(0, s)
        u = sim.u_field(0, 0)
    want = fp64_convolve(world, s[None])[0]
    err = float(np.abs(u - want).max())
    print("U field %s %d: max|err| = %.3e" % (path, side, err))
    assert err < (2e-5 if path == "bf16x3" else 2e-3), err


@pytest.mark.parametrize("path,tol", [("bf16x3", 1e-4), ("tf32", 5e-3)])
def test_tc_config2_teacher_forced(path, tol):
    world = configs.single_4096()
    with Sim(world, seed=configs.SEED_4096, path=path) as sim:
        s = sim.read_state(0)
        worst = 0.0
        for _ in range(2):
            sim.step(1)
            got = sim.read_state(0)
            worst = max(worst, float(np.abs(got - fp64_step(world, s)).max()))
            s = got
    print("config2 %s per-step max|err| vs FP64 = %.3e" % (path, worst))
    assert worst < tol, worst


@pytest.mark.parametrize("path", ["bf16x3", "tf32"])
def test_tc_batched_and_multichannel_run(path):
    worlds = configs.batched(24)
    with Sim(worlds, seed=0, path=path) as sim:
        for i, w in enumerate(worlds):
            sim.seed_patches(i, i, w.seed.patches)
        sim.step(3)
        before = [sim.read_state(i) for i in range(len(worlds))]
        sim.step(1)
        for i, w in enumerate(worlds):
            err = np.abs(sim.read_state(i) - fp64_step(w, before[i])).max()
            assert err < (1e-4 if path == "bf16x3" else 1e-2), (i, w.width, err)


def test_wait_timeout_reports_error_and_leaves_gpu_usable():
    """A tensor-core column pass whose first barrier wait gives up (the test hook sets its poll
    limit to zero, so it gives up before any MMA is issued) exits early -- after waiting, bounded,
    for its own DFT-matrix and tile loads and freeing its TMEM -- and raises the context's error
    flag: lenia_sync returns LENIA_ECUDA with a message, as the reference returns Err(String)
    (crates/auto-core/src/sim.rs:208-219).  Nothing is left waiting, so the same GPU then runs a
    fresh context to a one-step parity check against FP64, and the first context recovers too."""
    L = _lib.load()
    world = ag.World(256, 256, [ag.Kernel(radius=13.0)])
    rng = np.random.default_rng(7)
    s = rng.random((256, 256), dtype=np.float32)
    with Sim(world, path="bf16x3") as sim:
        sim.write_state(0, s)
        assert L.lenia_tc_set_wait_limit(sim._ctx, 1) == 0
        assert L.lenia_step(sim._ctx, 1) == 0
        rc = L.lenia_sync(sim._ctx)
        assert rc == _lib.ECUDA, rc
        msg = L.lenia_last_error(sim._ctx).decode()
        assert "gave up waiting" in msg, msg
        # the flag is cleared once reported; with the default limit the context steps correctly again
        assert L.lenia_tc_set_wait_limit(sim._ctx, 0) == 0
        sim.write_state(0, s)
        sim.step(1)
        assert L.lenia_sync(sim._ctx) == 0
        err_same = float(np.abs(sim.read_state(0) - fp64_step(world, s[None])).max())
    with Sim(world, path="bf16x3") as fresh:
        fresh.write_state(0, s)
        fresh.step(1)
        assert L.lenia_sync(fresh._ctx) == 0
        err_fresh = float(np.abs(fresh.read_state(0) - fp64_step(world, s[None])).max())
    print("after a forced wait timeout: same context %.3e, fresh context %.3e vs FP64" % (err_same, err_fresh))
    assert err_same < 1e-4 and err_fresh < 1e-4, (err_same, err_fresh)


def test_wait_limit_hook_rejected_without_tensor_cores():
    L = _lib.load()
    with Sim(ag.World(64, 64, [ag.Kernel(radius=8.0)]), path="fp32") as sim:
        assert L.lenia_tc_set_wait_limit(sim._ctx, 1) == _lib.ESTATE


@pytest.mark.parametrize("path,tol", [("bf16x3", 1e-4), ("tf32", 1e-2)])
@pytest.mark.parametrize("w,h", [(256, 256), (512, 512), (1024, 1024), (1024, 256), (256, 512), (512, 1024)])
def test_tc_row_pass_vs_fp64(path, tol, w, h):
    """The tensor-core row pass (inverse row DFT, growth / dt / clamp, forward row DFT as GEMMs) on
    the rows it serves, square and not: teacher-forced steps against the FP64 oracle with it on and
    off (the FP32 row pass), after every step of three.  The class reports which row pass it runs."""
    world = ag.World(w, h, [ag.Kernel(radius=min(13.0, min(w, h) / 4))])
    rng = np.random.default_rng(w * 7 + h)
    s0 = np.zeros((h, w), np.float32)
    s0[h // 4:3 * h // 4, w // 4:3 * w // 4] = rng.random((h // 2, w // 2), dtype=np.float32)
    errs = {}
    for on in (True, False):
        with Sim(world, path=path) as sim:
            sim.set_tc_rows(on)
            assert sim.shapes()[(w, h)]["tc_rows"] == (1 if on else 0)
            sim.write_state(0, s0)
            s = s0[None]
            worst = 0.0
            for _ in range(3):
                sim.step(1)
                got = sim.read_state(0)
                worst = max(worst, float(np.abs(got - fp64_step(world, s)).max()))
                s = got
            errs[on] = worst
            mass = float(s.mean())
    print("%s %dx%d per-step max|err| vs FP64: tensor-core rows %.3e, FP32 rows %.3e (mean state %.4f)" %
          (path, w, h, errs[True], errs[False], mass))
    assert errs[True] < tol and errs[False] < tol, errs
    assert 0.0 < mass < 1.0


def test_tc_row_pass_batched_many_steps():
    """The batched workload's tensor-core classes (256, 512, 1024) over 64 steps with the row pass on
    the tensor cores, checked teacher-forced against FP64 at the last step."""
    worlds = [w for w in configs.batched(96) if w.width in (256, 512, 1024)][:24]
    with Sim(worlds, seed=0, path="bf16x3") as sim:
        for i, w in enumerate(worlds):
            sim.seed_patches(i, i, w.seed.patches)
        sim.set_tc_rows(True)
        assert all(v["tc_rows"] == 1 for v in sim.shapes().values())
        sim.step(63)
        before = [sim.read_state(i) for i in range(len(worlds))]
        sim.step(1)
        worst, alive = 0.0, 0
        for i, w in enumerate(worlds):
            got = sim.read_state(i)
            worst = max(worst, float(np.abs(got - fp64_step(w, before[i])).max()))
            alive += int(got.mean() > 0)
    print("batched tensor-core classes, step 64: per-step max|err| vs FP64 %.3e, %d of %d worlds alive" %
          (worst, alive, len(worlds)))
    assert worst < 1e-4, worst
    assert alive > len(worlds) // 2


def test_tc_column_variants_bit_identical():
    """The tensor-core column pass's two variants (tile groups staged by bulk copies, or read from L2
    with more CTAs an SM) run the same arithmetic on the same values: bit-identical states after 8
    steps on batched worlds of every tensor-core column length, and within 1e-4 of FP64."""
    worlds = [w for w in configs.batched(96) if w.width in (256, 512, 1024)][:18]
    out = []
    for v in (0, 1):
        with Sim(worlds, seed=0, path="bf16x3") as sim:
            for i, w in enumerate(worlds):
                sim.seed_patches(i, i, w.seed.patches)
            sim.set_tc_variant(v)
            assert all(s["tc_column_variant"] == v for s in sim.shapes().values())
            sim.step(7)
            before = [sim.read_state(i) for i in range(len(worlds))]
            sim.step(1)
            out.append(sim.read_states().copy())
    assert np.array_equal(out[0], out[1])
    off = 0
    for i, w in enumerate(worlds):
        n = w.width * w.height
        err = float(np.abs(out[1][off:off + n].reshape(1, w.height, w.width) - fp64_step(w, before[i])).max())
        assert err < 1e-4, (i, err)
        off += n
