"""Sim: the engine context behind the reference's ``Sim`` interface (crates/auto-core/src/sim.rs).

``Sim(world_or_worlds, seed)`` mirrors ``Sim::new(&gpu, program, seed)`` (sim.rs:202-282),
``step(steps)`` mirrors ``Sim::step`` (sim.rs:297-309), ``read_field("state")`` and
``write_field("state", bytes)`` mirror sim.rs:560-595.  Several worlds may share one Sim; they
advance together in one set of launches.
"""
import ctypes
from typing import List, Sequence, Union

import numpy as np

from . import _lib
from ._lib import check, fptr
from .program import World


class Sim:
    def __init__(self, worlds: Union[World, Sequence[World]], seed: int = 1, path: Union[str, int] = "fp32"):
        self.worlds: List[World] = [worlds] if isinstance(worlds, World) else list(worlds)
        if not self.worlds:
            raise ValueError("need at least one world")
        self.path = _lib.PATHS[path] if isinstance(path, str) else int(path)
        self.seed = seed
        L = _lib.load()
        descs = (_lib.LeniaWorldDesc * len(self.worlds))(*[w.to_desc() for w in self.worlds])
        ctx = ctypes.c_void_p()
        check(L.lenia_create(descs, len(self.worlds), self.path, ctypes.byref(ctx)), None)
        self._ctx = ctx
        self._L = L
        self.run_init()

    # ------------------------------------------------------------------ lifecycle
    def close(self):
        if getattr(self, "_ctx", None):
            self._L.lenia_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc):
        return check(rc, self._ctx)

    # ------------------------------------------------------------------ the reference API
    def run_init(self):
        """Seed every world from its program's seed spec (sim.rs:286-294)."""
        for i, w in enumerate(self.worlds):
            s = w.seed
            if s.kind == "patches":
                self.seed_patches(i, self.seed, s.patches)
            elif s.kind == "tiles" and s.pattern is not None:
                self.seed_tiles(i, self.seed, s.pattern, s.spacing)
            elif s.kind == "discs":
                self.seed_rule(i, self.seed, _lib.SEED_SL_DISCS)
            elif s.kind == "blocks":
                self.seed_rule(i, self.seed, _lib.SEED_MNCA_BLOCKS)

    @property
    def tick(self) -> int:
        t = ctypes.c_uint64()
        self._check(self._L.lenia_tick(self._ctx, ctypes.byref(t)))
        return int(t.value)

    def step(self, steps: int) -> int:
        """Advance every world by ``steps``; returns generations advanced (asynchronous)."""
        self._check(self._L.lenia_step(self._ctx, int(steps)))
        return int(steps)

    def step_timed(self, steps: int) -> float:
        """Advance and block; device milliseconds of the steps (CUDA events on the engine stream)."""
        ms = ctypes.c_float()
        self._check(self._L.lenia_step_timed(self._ctx, int(steps), ctypes.byref(ms)))
        return float(ms.value)

    def wait(self):
        self._check(self._L.lenia_sync(self._ctx))

    def read_field(self, name: str, world: int = 0) -> bytes:
        if name != "state":
            raise KeyError("known field: state")
        return self.read_state(world).tobytes()

    def write_field(self, name: str, data: bytes, world: int = 0):
        if name != "state":
            raise KeyError("known field: state")
        w = self.worlds[world]
        self.write_state(world, np.frombuffer(data, np.float32).reshape(w.channels, w.height, w.width))

    # ------------------------------------------------------------------ arrays
    def read_state(self, world: int = 0) -> np.ndarray:
        w = self.worlds[world]
        out = np.empty((w.channels, w.height, w.width), np.float32)
        self._check(self._L.lenia_read_state(self._ctx, world, fptr(out), out.size))
        return out

    def read_states(self, out: np.ndarray = None) -> np.ndarray:
        """Every world's state, back to back in world order, as one flat float32 array."""
        n = sum(w.channels * w.height * w.width for w in self.worlds)
        if out is None:
            out = np.empty(n, np.float32)
        self._check(self._L.lenia_read_states(self._ctx, fptr(out), out.size))
        return out

    def write_states(self, states: np.ndarray):
        """Write every world's state from one flat array (world order, as read_states returns)."""
        a = np.ascontiguousarray(states, np.float32).ravel()
        self._check(self._L.lenia_write_states(self._ctx, fptr(a), a.size))
        self.wait()

    def write_states_async(self, states: np.ndarray):
        """write_states without blocking: `states` (contiguous float32, page-locked for the copy to
        overlap the steps) must stay untouched until wait()."""
        if states.dtype != np.float32 or not states.flags.c_contiguous:
            raise ValueError("write_states_async needs a contiguous float32 array that outlives the copy")
        self._check(self._L.lenia_write_states_async(self._ctx, fptr(states), states.size))

    def read_states_async(self, out: np.ndarray):
        """read_states without blocking into `out` (contiguous float32, page-locked for the copy to
        overlap the steps), complete after wait()."""
        if out.dtype != np.float32 or not out.flags.c_contiguous:
            raise ValueError("read_states_async needs a contiguous float32 array")
        self._check(self._L.lenia_read_states_async(self._ctx, fptr(out), out.size))

    def write_state(self, world: int, state: np.ndarray):
        a = np.ascontiguousarray(state, np.float32).ravel()
        self._check(self._L.lenia_write_state(self._ctx, world, fptr(a), a.size))
        self.wait()

    def seed_patches(self, world: int, seed: int, patches):
        p = np.ascontiguousarray(np.asarray(patches, np.int32).reshape(-1, 4))
        self._check(self._L.lenia_seed_patches(self._ctx, world, seed,
                                               p.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), len(p)))

    def seed_tiles(self, world: int, seed: int, pattern, spacing: int = 64):
        pat = np.ascontiguousarray(pattern, np.float32)
        self._check(self._L.lenia_seed_tiles(self._ctx, world, seed, fptr(pat), pat.shape[1], pat.shape[0], spacing))

    def seed_rule(self, world: int, seed: int, kind: int):
        """SmoothLife discs (_lib.SEED_SL_DISCS) or MNCA blocks (_lib.SEED_MNCA_BLOCKS)."""
        self._check(self._L.lenia_seed_rule(self._ctx, world, seed, kind))

    def render(self, world: int = 0, out_w: int = 256, out_h: int = 256, origin=(0.0, 0.0), scale: float = 1.0,
               samples: int = 2, palette: int = 0, channel: int = 0) -> np.ndarray:
        """Headless view (sim.rs:17-41): (out_h, out_w, 4) uint8 RGBA."""
        out = np.zeros((out_h, out_w, 4), np.uint8)
        self._check(self._L.lenia_render(self._ctx, world, channel, float(origin[0]), float(origin[1]), float(scale),
                                         samples, out_w, out_h, palette, out.ctypes.data_as(ctypes.c_void_p)))
        return out

    def u_field(self, world: int = 0, kernel: int = 0) -> np.ndarray:
        w = self.worlds[world]
        out = np.empty((w.height, w.width), np.float32)
        self._check(self._L.lenia_read_field_u(self._ctx, world, kernel, fptr(out), out.size))
        return out

    def spectrum(self, world: int = 0, channel: int = 0) -> np.ndarray:
        w = self.worlds[world]
        out = np.empty((w.height, w.width // 2 + 1, 2), np.float32)
        self._check(self._L.lenia_read_spectrum(self._ctx, world, channel, fptr(out), out.size))
        return out[..., 0] + 1j * out[..., 1]

    def stats(self) -> np.ndarray:
        """(mass, centroid x, centroid y) per world."""
        out = np.empty((len(self.worlds), 3), np.float32)
        self._check(self._L.lenia_world_stats(self._ctx, fptr(out), out.size))
        return out

    @property
    def cells_per_step(self) -> int:
        v = ctypes.c_uint64()
        self._check(self._L.lenia_cells_per_step(self._ctx, ctypes.byref(v)))
        return int(v.value)

    @property
    def memory_bytes(self) -> int:
        v = ctypes.c_uint64()
        self._check(self._L.lenia_memory_bytes(self._ctx, ctypes.byref(v)))
        return int(v.value)

    def autotune(self):
        self._check(self._L.lenia_autotune(self._ctx))

    def variants(self):
        """{(width, height): (column variant, row variant)} for every size class."""
        n = ctypes.c_size_t(0)
        self._check(self._L.lenia_class_variants(self._ctx, None, 0, ctypes.byref(n)))
        out = (ctypes.c_int32 * (4 * n.value))()
        self._check(self._L.lenia_class_variants(self._ctx, out, 4 * n.value, ctypes.byref(n)))
        return {(out[4 * i], out[4 * i + 1]): (out[4 * i + 2], out[4 * i + 3]) for i in range(n.value)}

    def shapes(self):
        """{(width, height): {...}} for every size class: launch variants, chunks (L2-resident runs of
        worlds), worlds, chunk budget (MiB, 0 = one chunk), rows per row-pass item and whether the class runs
        the cluster-resident step, whether its row pass runs on the tensor cores, its tensor-core column
        pass variant (-1: none), its persistent step's launch variant (-1: it does not run it), and the
        concurrent lanes its chunks run on."""
        n = ctypes.c_size_t(0)
        self._check(self._L.lenia_class_shapes(self._ctx, None, 0, ctypes.byref(n)))
        out = (ctypes.c_int32 * (14 * n.value))()
        self._check(self._L.lenia_class_shapes(self._ctx, out, 14 * n.value, ctypes.byref(n)))
        keys = ("column_variant", "row_variant", "chunks", "worlds", "chunk_budget_mib", "rows_per_row_item",
                "resident", "resident_variant", "tc_rows", "tc_column_variant", "persistent", "lanes")
        return {(out[14 * i], out[14 * i + 1]): dict(zip(keys, out[14 * i + 2:14 * i + 14])) for i in range(n.value)}

    def set_resident(self, on: bool, variant: int = -1):
        """Cluster-resident step on or off where it applies, optionally in launch variant `variant`
        (see lenia_set_resident)."""
        self._check(self._L.lenia_set_resident(self._ctx, (2 + variant if variant >= 0 else 1) if on else 0))

    def set_tc_rows(self, on: bool):
        """Tensor-core row pass on or off on the TF32 / BF16X3 paths (see lenia_set_tc_rows)."""
        self._check(self._L.lenia_set_tc_rows(self._ctx, 1 if on else 0))

    def set_persistent(self, on: bool, variant: int = -1):
        """Persistent step on or off where it applies, optionally in launch variant `variant` (see
        lenia_set_persistent)."""
        self._check(self._L.lenia_set_persistent(self._ctx, (2 + variant if variant >= 0 else 1) if on else 0))

    def set_persist_wait_limit(self, polls_plus_one: int):
        """Test hook: the persistent step's wait limit + 1 (0: the default; 1: every dependency wait
        gives up at once; see lenia_persist_set_wait_limit)."""
        self._check(self._L.lenia_persist_set_wait_limit(self._ctx, int(polls_plus_one)))

    def set_tc_variant(self, variant: int):
        """Tensor-core column pass variant of every class (see lenia_set_tc_variant)."""
        self._check(self._L.lenia_set_tc_variant(self._ctx, int(variant)))

    def set_branch_split(self, cells: int, each: bool = False):
        """Classes of at most `cells` cells a world on side graph branches, one after another or each
        on its own (see lenia_set_branch_split)."""
        self._check(self._L.lenia_set_branch_split(self._ctx, int(cells), 1 if each else 0))

    @property
    def branch_split(self):
        """(cells, each) of the step graph's branch split."""
        c, e = ctypes.c_int64(), ctypes.c_int32()
        self._check(self._L.lenia_branch_split(self._ctx, ctypes.byref(c), ctypes.byref(e)))
        return int(c.value), bool(e.value)

    def set_chunk_budget(self, mib: int):
        """Pin every size class's chunk budget in MiB (see lenia_set_chunk_budget); 0 = one chunk."""
        self._check(self._L.lenia_set_chunk_budget(self._ctx, int(mib)))

    def set_chunk_lanes(self, lanes: int):
        """Pin every size class's chunk lanes, 1..4 (see lenia_set_chunk_lanes)."""
        self._check(self._L.lenia_set_chunk_lanes(self._ctx, int(lanes)))

    def set_variants(self, column: int = -1, row: int = -1):
        """Pin every size class's launch variants (see lenia_set_variants); -1 keeps one."""
        self._check(self._L.lenia_set_variants(self._ctx, int(column), int(row)))

    def profile(self, steps: int = 10):
        """Event-timed (column ms, row ms, step ms) per step."""
        out = np.zeros(3, np.float32)
        self._check(self._L.lenia_profile_step(self._ctx, int(steps), fptr(out)))
        return out

    def profile_classes(self, steps: int = 5):
        """Per size class: {(width, height): (column ms, row ms, graph ms)} per step, each class timed
        alone: its column and row launches one at a time, and the class as the step graph runs it."""
        n = ctypes.c_size_t()
        self._check(self._L.lenia_profile_classes(self._ctx, int(steps), None, 0, ctypes.byref(n)))
        out = np.zeros(5 * n.value, np.float32)
        self._check(self._L.lenia_profile_classes(self._ctx, int(steps), fptr(out), out.size, ctypes.byref(n)))
        return {(int(out[5 * i]), int(out[5 * i + 1])): tuple(float(x) for x in out[5 * i + 2:5 * i + 5])
                for i in range(n.value)}
