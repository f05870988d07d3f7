"""CPU oracle for the Lenia-family FFT step.  TEST INFRASTRUCTURE ONLY.

Two checkers live here; only tests/, the smoke check and bench.py's CPU-baseline leg use them,
and the shipped library never does:

* ``RefF32`` -- ctypes front end of oracle/lenia_oracle.c, the f32 restatement of the reference's
  pass sequence (crates/auto-core/src/automata/spectral.rs:14-64, 75-83, 150-181, 199-264,
  337-345; program.rs:140-147).  Power-of-two grids, one channel, 1-3 kernels, as the reference.
* ``fp64_*`` -- the same mathematics in float64 with numpy's FFT, generalised to multi-shell
  kernels, several channels, any grid size and per-world parameters (no reference code exists
  for those; the multi-shell kernel follows Chan's Lenia definition).

World/kernel descriptions are duck-typed: any object with the attributes of
``auto_gb300.program.World`` / ``Kernel`` works.
"""
import ctypes
import os

import numpy as np

from . import build as _build

try:  # multi-threaded float64 FFTs when scipy is present; numpy's otherwise (same results)
    import scipy.fft as _sfft

    def _rfft2(a):
        return _sfft.rfft2(a, workers=-1)

    def _irfft2(a, s):
        return _sfft.irfft2(a, s=s, workers=-1)
except ImportError:  # pragma: no cover
    def _rfft2(a):
        return np.fft.rfft2(a)

    def _irfft2(a, s):
        return np.fft.irfft2(a, s=s)

SHAPE_LENIA, SHAPE_SL_INNER, SHAPE_SL_OUTER, SHAPE_RING = 0, 1, 2, 3
RULE_LENIA, RULE_SMOOTHLIFE, RULE_MNCA = 0, 1, 2


class _OrcKernel(ctypes.Structure):
    _fields_ = [("shape", ctypes.c_int32), ("radius", ctypes.c_float), ("nshells", ctypes.c_int32),
                ("beta", ctypes.c_float * 3), ("lo", ctypes.c_float), ("hi", ctypes.c_float)]


class _OrcRule(ctypes.Structure):
    _fields_ = [("rule", ctypes.c_int32), ("mu", ctypes.c_float), ("sigma", ctypes.c_float),
                ("dt", ctypes.c_float)]


def _fptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def _orc_kernel(k):
    ok = _OrcKernel()
    ok.shape = int(k.shape)
    ok.radius = float(k.radius)
    beta = list(getattr(k, "beta", [1.0]) or [1.0])
    ok.nshells = len(beta)
    for i, b in enumerate(beta[:3]):
        ok.beta[i] = float(b)
    ok.lo = float(getattr(k, "lo", 0.0))
    ok.hi = float(getattr(k, "hi", 0.0))
    return ok


class RefF32:
    """The reference's f32 step, restated in C (see oracle/lenia_oracle.c)."""

    def __init__(self, threads: int = 0):
        path = _build.build()
        self.lib = ctypes.CDLL(path)
        L = self.lib
        L.orc_rand3.restype = ctypes.c_uint32
        L.orc_rand3.argtypes = [ctypes.c_uint32] * 3
        L.orc_pcg.restype = ctypes.c_uint32
        L.orc_pcg.argtypes = [ctypes.c_uint32]
        L.orc_unit_f.restype = ctypes.c_float
        L.orc_unit_f.argtypes = [ctypes.c_uint32]
        L.orc_kernel_sum.restype = ctypes.c_float
        L.orc_kernel_sum.argtypes = [ctypes.POINTER(_OrcKernel)]
        L.orc_kernel_spatial.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(_OrcKernel),
                                         ctypes.POINTER(ctypes.c_float)]
        L.orc_kernel_spectrum.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_float),
                                          ctypes.POINTER(ctypes.c_float), ctypes.c_int]
        L.orc_step.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_float),
                               ctypes.POINTER(_OrcRule), ctypes.POINTER(ctypes.c_float),
                               ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float),
                               ctypes.c_int, ctypes.c_int]
        L.orc_direct_lenia_step.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.c_int,
                                            ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                            ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)]
        L.orc_seed_tiles.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_uint32, ctypes.POINTER(ctypes.c_float),
                                     ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_float)]
        L.orc_seed_patches.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_uint32,
                                       ctypes.POINTER(ctypes.c_int32), ctypes.c_int, ctypes.POINTER(ctypes.c_float)]
        L.orc_seed_sl_discs.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_uint32, ctypes.POINTER(ctypes.c_float)]
        L.orc_seed_mnca_blocks.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_uint32, ctypes.POINTER(ctypes.c_float)]
        L.orc_render.argtypes = [ctypes.POINTER(ctypes.c_float), ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                 ctypes.c_float, ctypes.c_float, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                 ctypes.c_void_p]
        self.threads = threads or (os.cpu_count() or 1)

    # RNG (program.rs:140-147)
    def rand3(self, a, b, c):
        return int(self.lib.orc_rand3(a, b, c))

    def unit_f(self, r):
        return float(self.lib.orc_unit_f(r))

    def kernel_sum(self, k):
        ok = _orc_kernel(k)
        return float(self.lib.orc_kernel_sum(ctypes.byref(ok)))

    def kernel_spatial(self, w, h, k):
        out = np.zeros((h, w), np.float32)
        ok = _orc_kernel(k)
        self.lib.orc_kernel_spatial(w, h, ctypes.byref(ok), _fptr(out))
        return out

    def kernel_spectrum(self, w, h, k):
        sp = self.kernel_spatial(w, h, k)
        out = np.zeros((h, w, 2), np.float32)
        rc = self.lib.orc_kernel_spectrum(w, h, _fptr(sp), _fptr(out), self.threads)
        if rc != 0:
            raise ValueError("FFT grids must be powers of two")
        return out

    def spectra(self, world):
        return np.stack([self.kernel_spectrum(world.width, world.height, k) for k in world.kernels])

    def step(self, world, state, steps=1, spectra=None, return_conv=False, threads=None):
        """Advance a single-channel world by ``steps`` f32 steps; state is (h, w) float32."""
        w, h = world.width, world.height
        if world.channels != 1 or not 1 <= len(world.kernels) <= 3:
            raise ValueError("the reference step handles one channel and 1-3 kernels")
        spectra = self.spectra(world) if spectra is None else spectra
        spectra = np.ascontiguousarray(spectra, np.float32)
        rule = _OrcRule()
        rule.rule = int(world.rule)
        k0 = world.kernels[0]
        rule.mu, rule.sigma, rule.dt = float(k0.mu), float(k0.sigma), float(world.dt)
        s_in = np.ascontiguousarray(state, np.float32).reshape(h, w)
        s_out = np.zeros((h, w), np.float32)
        conv = np.zeros((len(world.kernels), h, w), np.float32)
        rc = self.lib.orc_step(w, h, len(world.kernels), _fptr(spectra), ctypes.byref(rule), _fptr(s_in),
                               _fptr(s_out), _fptr(conv), int(steps), int(threads or self.threads))
        if rc != 0:
            raise ValueError("orc_step failed (%d)" % rc)
        return (s_out, conv) if return_conv else s_out

    def direct_lenia_step(self, state, radius=13.0, reach=14, mu=0.15, sigma=0.015, dt=0.1):
        """crates/auto-core/tests/automata.rs:300-362 (f64 direct convolution, one step)."""
        h, w = state.shape
        s = np.ascontiguousarray(state, np.float32)
        out = np.zeros_like(s)
        self.lib.orc_direct_lenia_step(w, h, radius, reach, mu, sigma, dt, _fptr(s), _fptr(out))
        return out

    def seed_tiles(self, w, h, seed, pattern, spacing=64):
        pat = np.ascontiguousarray(pattern, np.float32)
        out = np.zeros((h, w), np.float32)
        self.lib.orc_seed_tiles(w, h, seed, _fptr(pat), pat.shape[1], pat.shape[0], spacing, _fptr(out))
        return out

    def seed_sl_discs(self, w, h, seed):
        out = np.zeros((h, w), np.float32)
        self.lib.orc_seed_sl_discs(w, h, seed, _fptr(out))
        return out

    def seed_mnca_blocks(self, w, h, seed):
        out = np.zeros((h, w), np.float32)
        self.lib.orc_seed_mnca_blocks(w, h, seed, _fptr(out))
        return out

    def render(self, state, out_w, out_h, origin=(0.0, 0.0), scale=1.0, samples=2, palette=0):
        s = np.ascontiguousarray(state, np.float32)
        h, w = s.shape
        out = np.zeros((out_h, out_w, 4), np.uint8)
        self.lib.orc_render(_fptr(s), w, h, float(origin[0]), float(origin[1]), float(scale), samples, out_w, out_h,
                            palette, out.ctypes.data_as(ctypes.c_void_p))
        return out

    def seed_patches(self, w, h, seed, patches):
        p = np.ascontiguousarray(np.asarray(patches, np.int32).reshape(-1, 4))
        out = np.zeros((h, w), np.float32)
        self.lib.orc_seed_patches(w, h, seed, p.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), len(p), _fptr(out))
        return out


# ----------------------------------------------------------------------------- FP64 oracle

def _lenia_core64(q):
    out = np.zeros_like(q)
    m = (q > 0) & (q < 1)
    qm = q[m]
    out[m] = np.exp(4.0 - 1.0 / (qm * (1.0 - qm)))
    return out


def fp64_shape(k, r):
    """Kernel shape in float64 (spectral.rs:288-295, 356-359, 427-433; shells per Chan)."""
    r = np.asarray(r, np.float64)
    shape = int(k.shape)
    if shape == SHAPE_LENIA:
        beta = list(getattr(k, "beta", [1.0]) or [1.0])
        B = len(beta)
        q = r / float(k.radius)
        if B == 1:
            return beta[0] * _lenia_core64(q)
        inside = (q > 0) & (q < 1)
        bq = B * q
        idx = np.clip(np.floor(bq).astype(np.int64), 0, B - 1)
        vals = np.asarray(beta, np.float64)[idx] * _lenia_core64(bq - idx)
        return np.where(inside, vals, 0.0)
    if shape == SHAPE_SL_INNER:
        ri, aa = float(k.radius) / 3.0, 0.5
        return np.clip((ri + aa - r) / (2 * aa), 0.0, 1.0)
    if shape == SHAPE_SL_OUTER:
        ra, ri, aa = float(k.radius), float(k.radius) / 3.0, 0.5
        return np.clip((ra + aa - r) / (2 * aa), 0.0, 1.0) * np.clip((r - ri + aa) / (2 * aa), 0.0, 1.0)
    if shape == SHAPE_RING:
        return ((r >= float(k.lo)) & (r < float(k.hi))).astype(np.float64)
    raise ValueError("unknown shape %r" % shape)


def fp64_kernel_spatial(w, h, k):
    """Kernel at min-image torus distance, divided by its float64 sum (spectral.rs:150-171)."""
    x = np.arange(w)
    y = np.arange(h)
    dx = np.minimum(x, w - x).astype(np.float64)
    dy = np.minimum(y, h - y).astype(np.float64)
    r = np.sqrt(dx[None, :] ** 2 + dy[:, None] ** 2)
    v = fp64_shape(k, r)
    return v / v.sum()


def fp64_khat(w, h, k):
    """Real, even kernel spectrum (h, w//2+1) in float64.  The imaginary part is zero up to
    rounding because the min-image kernel is even in both axes."""
    return _rfft2(fp64_kernel_spatial(w, h, k)).real


def fp64_khats(world):
    return [fp64_khat(world.width, world.height, k) for k in world.kernels]


def fp64_growth(u, mu, sigma):
    d = (u - mu) / sigma
    return 2.0 * np.exp(-0.5 * d * d) - 1.0


def fp64_convolve(world, state, khats=None):
    """U_k for every kernel: state (C, h, w) -> (K, h, w) float64."""
    w, h = world.width, world.height
    khats = fp64_khats(world) if khats is None else khats
    st = np.asarray(state, np.float64).reshape(world.channels, h, w)
    specs = [_rfft2(st[c]) for c in range(world.channels)]
    return np.stack([_irfft2(specs[int(k.src)] * khats[i], s=(h, w))
                     for i, k in enumerate(world.kernels)])


def fp64_update(world, state, conv):
    st = np.asarray(state, np.float64).reshape(world.channels, conv.shape[1], conv.shape[2])
    rule = int(world.rule)
    if rule == RULE_LENIA:
        acc = np.zeros_like(st)
        for i, k in enumerate(world.kernels):
            acc[int(k.dst)] += float(k.weight) * fp64_growth(conv[i], float(k.mu), float(k.sigma))
        return np.clip(st + float(world.dt) * acc, 0.0, 1.0)
    if rule == RULE_SMOOTHLIFE:
        B1, B2, D1, D2, AN, AM, DT = 0.278, 0.365, 0.267, 0.445, 0.028, 0.147, 0.1
        sig = lambda x, a, al: 1.0 / (1.0 + np.exp((a - x) * 4.0 / al))
        m = sig(conv[0], 0.5, AM)
        lo, hi = B1 * (1 - m) + D1 * m, B2 * (1 - m) + D2 * m
        target = sig(conv[1], lo, AN) * (1.0 - sig(conv[1], hi, AN))
        return np.clip(st + DT * (2.0 * target - 1.0), 0.0, 1.0)
    if rule == RULE_MNCA:
        c0, c1 = conv[0], conv[1]
        o = st[0].copy()
        band = lambda v, lo, hi: (v >= lo) & (v <= hi)
        o = np.where(band(c0, 0.210, 0.220), 1.0, o)
        o = np.where(band(c0, 0.350, 0.500), 0.0, o)
        o = np.where(band(c0, 0.750, 0.850), 0.0, o)
        o = np.where(band(c0, 0.120, 0.150), 0.0, o)
        o = np.where(band(c1, 0.100, 0.280), 0.0, o)
        o = np.where(band(c1, 0.430, 0.550), 1.0, o)
        return o[None]
    raise ValueError("unknown rule %r" % rule)


def fp64_step(world, state, steps=1, khats=None):
    """Advance (C, h, w) state by ``steps`` float64 steps."""
    khats = fp64_khats(world) if khats is None else khats
    st = np.asarray(state, np.float64).reshape(world.channels, world.height, world.width)
    for _ in range(steps):
        st = fp64_update(world, st, fp64_convolve(world, st, khats))
    return st
