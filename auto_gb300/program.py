"""World descriptions and the automaton registry, mirroring the reference's plugin API.

The reference describes an automaton as an ``Entry`` (crates/auto-core/src/automata/mod.rs:14-27)
whose ``build(w, h)`` returns a ``Program`` (program.rs:102-129); the spectral ones are built by
``spectral::lenia / smoothlife / mnca_shaped`` (spectral.rs:286-510).  Here a ``World`` carries the
same information as data -- grid, kernels, growth parameters -- so that many worlds with their
own parameters can share one engine context.
"""
from dataclasses import dataclass, field
from typing import Callable, List, Optional, Sequence, Tuple

from . import _lib
from ._lib import (RULE_LENIA, RULE_MNCA, RULE_SMOOTHLIFE, SHAPE_LENIA, SHAPE_RING, SHAPE_SL_INNER,
                   SHAPE_SL_OUTER)

M32 = 0xFFFFFFFF


def pcg(v: int) -> int:
    """PCG hash (program.rs:140-144)."""
    s = (v * 747796405 + 2891336453) & M32
    w = (((s >> ((s >> 28) + 4)) ^ s) * 277803737) & M32
    return ((w >> 22) ^ w) & M32


def rand3(a: int, b: int, c: int) -> int:
    """program.rs:145."""
    return pcg(pcg(pcg(a & M32) ^ (b & M32)) ^ (c & M32))


def unit_f(r: int) -> float:
    """program.rs:146 (as float64 of the f32 value)."""
    import numpy as np
    return float(np.float32(np.float32(r) * np.float32(1.0 / 4294967296.0)))


@dataclass
class Kernel:
    shape: int = SHAPE_LENIA
    radius: float = 13.0
    beta: List[float] = field(default_factory=lambda: [1.0])
    lo: float = 0.0
    hi: float = 0.0
    src: int = 0
    dst: int = 0
    mu: float = 0.15
    sigma: float = 0.015
    weight: float = 1.0


@dataclass
class Seed:
    """How a world's initial state is made on the device (the reference's seed pass)."""
    kind: str = "none"                    # "none" | "patches" | "tiles" | "discs" | "blocks"
    patches: List[Tuple[int, int, int, int]] = field(default_factory=list)
    spacing: int = 64
    pattern: Optional[object] = None      # 2-D float array for "tiles"


@dataclass
class World:
    """One world: the data of a reference ``Program`` for a spectral automaton."""
    width: int
    height: int
    kernels: List[Kernel]
    channels: int = 1
    dt: float = 0.1
    rule: int = RULE_LENIA
    id: str = "lenia"
    seed: Seed = field(default_factory=Seed)

    @property
    def cells_per_step(self) -> int:
        """Program::cells_per_step (spectral.rs:280) times the channel count."""
        return self.width * self.height * self.channels

    def to_desc(self) -> _lib.LeniaWorldDesc:
        if len(self.kernels) > _lib.MAX_KERNELS:
            raise ValueError("at most %d kernels" % _lib.MAX_KERNELS)
        d = _lib.LeniaWorldDesc()
        d.width, d.height, d.channels = self.width, self.height, self.channels
        d.nkernels, d.rule, d.dt = len(self.kernels), self.rule, self.dt
        for i, k in enumerate(self.kernels):
            kk = d.kernels[i]
            kk.shape, kk.radius = k.shape, k.radius
            beta = list(k.beta) or [1.0]
            kk.nshells = len(beta)
            for j, b in enumerate(beta[:3]):
                kk.beta[j] = b
            kk.ring_lo, kk.ring_hi = k.lo, k.hi
            kk.src, kk.dst, kk.mu, kk.sigma, kk.weight = k.src, k.dst, k.mu, k.sigma, k.weight
        return d


# ----------------------------------------------------------------------------- the registry

def lenia(w: int, h: int, radius: float = 13.0, pattern=None) -> World:
    """spectral.rs:286-352: ring kernel of radius R, mu 0.15, sigma 0.015, dt 0.1; seeded with a
    20x20 creature in random 64-cell tiles (the caller supplies the creature)."""
    seed = Seed(kind="tiles", spacing=64, pattern=pattern) if pattern is not None else Seed()
    return World(w, h, [Kernel(SHAPE_LENIA, radius, [1.0], mu=0.15, sigma=0.015)], dt=0.1, rule=RULE_LENIA,
                 id="lenia", seed=seed)


def smoothlife(w: int, h: int, ra: float = 21.0) -> World:
    """spectral.rs:355-415: inner disc ra/3 and outer ring, Rafler's transition."""
    return World(w, h, [Kernel(SHAPE_SL_INNER, ra), Kernel(SHAPE_SL_OUTER, ra)], rule=RULE_SMOOTHLIFE,
                 id="smoothlife", seed=Seed("discs"))


MNCA_RINGS = (12.0, 18.0, 3.0, 8.0)  # spectral.rs:423


def mnca_shaped(w: int, h: int, rings: Sequence[float] = MNCA_RINGS) -> World:
    """spectral.rs:426-480: two hard rings [inner0, outer0, inner1, outer1]."""
    return World(w, h, [Kernel(SHAPE_RING, lo=rings[0], hi=rings[1]), Kernel(SHAPE_RING, lo=rings[2], hi=rings[3])],
                 rule=RULE_MNCA, id="mnca", seed=Seed("blocks"))


def mnca(w: int, h: int) -> World:
    return mnca_shaped(w, h, MNCA_RINGS)


@dataclass
class Entry:
    """automata::Entry (mod.rs:14-27)."""
    id: str
    name: str
    blurb: str
    default_size: Tuple[int, int]
    needs_pot: bool
    width_step: int
    build: Callable[[int, int], World]


LENIA = Entry("lenia", "Lenia", "Continuous life. Each cell senses a ring of radius 13 through an FFT.",
              (2048, 1024), False, 1, lambda w, h: lenia(w, h, 13.0))
SMOOTHLIFE = Entry("smoothlife", "SmoothLife", "Rafler's continuous Game of Life: an inner disc and an outer ring.",
                   (2048, 1024), False, 1, lambda w, h: smoothlife(w, h, 21.0))
MNCA = Entry("mnca", "Multiple Neighbourhood CA", "Threshold bands on several neighbourhoods at once.",
             (2048, 1024), False, 1, mnca)
ALL = [LENIA, SMOOTHLIFE, MNCA]


def find(id: str) -> Optional[Entry]:
    """automata::find (mod.rs:48-50)."""
    for e in ALL:
        if e.id == id:
            return e
    return None


def _next_fft_size(n: int) -> int:
    """Smallest supported side >= n: 2^a or 3*2^a (the reference accepts powers of two only)."""
    best = None
    p = 32
    while p <= 8192:
        for c in (p, 3 * p // 2 if p >= 64 else None):
            if c and c >= n and (best is None or c < best):
                best = c
        p *= 2
    return best or n


def fit_size(entry: Entry, w: int, h: int) -> Tuple[int, int]:
    """automata::fit_size (mod.rs:52-62): round to a size the engine accepts."""
    if entry.needs_pot:
        return 1 << max(0, (w - 1).bit_length()), 1 << max(0, (h - 1).bit_length())
    return _next_fft_size(w), _next_fft_size(h)


def build(id: str, w: int, h: int) -> Optional[World]:
    """automata::build (mod.rs:65-95) for the spectral automata, including ``mnca.lo,hi,lo,hi``."""
    e = find(id)
    if e is not None:
        fw, fh = fit_size(e, w, h)
        return e.build(fw, fh)
    if id.startswith("mnca."):
        v = [float(p) for p in id[5:].split(",") if p]
        return mnca_shaped(_next_fft_size(w), _next_fft_size(h), v)
    return None
