"""ctypes binding of include/lenia_gb300.h.

The library is built in-tree (auto_gb300/_build/liblenia_gb300.so) by auto_gb300/build.py.  There
is no fallback: if the library is missing or fails to load, every engine call raises.
"""
import ctypes
import os

MAX_KERNELS = 16
MAX_CHANNELS = 4

OK, EINVAL, ESIZE, ENOMEM, ECUDA, ENODEV, ESTATE = 0, -1, -2, -3, -4, -5, -6
SHAPE_LENIA, SHAPE_SL_INNER, SHAPE_SL_OUTER, SHAPE_RING = 0, 1, 2, 3
RULE_LENIA, RULE_SMOOTHLIFE, RULE_MNCA = 0, 1, 2
PATH_FP32, PATH_TF32, PATH_BF16X3, PATH_RADIX2 = 0, 1, 2, 3
SELFTEST_A_MN = 0x100  # lenia_tc_selftest: A in the MN-major layout
PATHS = {"fp32": PATH_FP32, "tf32": PATH_TF32, "bf16x3": PATH_BF16X3, "radix2": PATH_RADIX2}

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_build", "liblenia_gb300.so")

# Every function the header declares, for the export check.
EXPORTS = [
    "lenia_last_error", "lenia_create", "lenia_destroy", "lenia_write_state", "lenia_read_state",
    "lenia_write_state_device", "lenia_read_state_device", "lenia_write_states", "lenia_read_states", "lenia_write_states_async", "lenia_read_states_async", "lenia_step", "lenia_step_timed", "lenia_sync",
    "lenia_tick", "lenia_seed_tiles", "lenia_seed_patches", "lenia_cells_per_step", "lenia_memory_bytes",
    "lenia_read_field_u", "lenia_read_spectrum", "lenia_world_stats", "lenia_autotune", "lenia_set_variants", "lenia_class_variants", "lenia_class_shapes", "lenia_set_chunk_budget", "lenia_set_chunk_lanes", "lenia_set_resident", "lenia_set_persistent", "lenia_set_tc_rows", "lenia_set_tc_variant", "lenia_set_branch_split", "lenia_branch_split", "lenia_profile_step", "lenia_profile_classes",
    "lenia_kernel_spectrum", "lenia_tc_selftest", "lenia_tc_set_wait_limit", "lenia_persist_set_wait_limit", "lenia_step_noalloc",
    "lenia_mlp_create", "lenia_mlp_destroy", "lenia_mlp_param_count", "lenia_mlp_set_params",
    "lenia_mlp_get_params", "lenia_mlp_gradients", "lenia_mlp_train_step", "lenia_mlp_predict",
    "lenia_seed_rule", "lenia_render",
]
SEED_SL_DISCS, SEED_MNCA_BLOCKS = 1, 2
PALETTE_LENIA, PALETTE_SMOOTHLIFE, PALETTE_MNCA = 0, 1, 2


class LeniaKernel(ctypes.Structure):
    _fields_ = [("shape", ctypes.c_int32), ("radius", ctypes.c_float), ("nshells", ctypes.c_int32),
                ("beta", ctypes.c_float * 3), ("ring_lo", ctypes.c_float), ("ring_hi", ctypes.c_float),
                ("src", ctypes.c_int32), ("dst", ctypes.c_int32), ("mu", ctypes.c_float),
                ("sigma", ctypes.c_float), ("weight", ctypes.c_float)]


class LeniaWorldDesc(ctypes.Structure):
    _fields_ = [("width", ctypes.c_uint32), ("height", ctypes.c_uint32), ("channels", ctypes.c_uint32),
                ("nkernels", ctypes.c_uint32), ("rule", ctypes.c_int32), ("dt", ctypes.c_float),
                ("kernels", LeniaKernel * MAX_KERNELS)]


class LeniaError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (code %d)" % (msg, code))
        self.code = code


_lib = None

_c_float_p = ctypes.POINTER(ctypes.c_float)


def _declare(L):
    vp = ctypes.c_void_p
    sz = ctypes.c_size_t
    i32 = ctypes.c_int32
    u32 = ctypes.c_uint32
    L.lenia_last_error.restype = ctypes.c_char_p
    L.lenia_last_error.argtypes = [vp]
    sig = {
        "lenia_create": [ctypes.POINTER(LeniaWorldDesc), i32, i32, ctypes.POINTER(vp)],
        "lenia_destroy": [vp],
        "lenia_write_state": [vp, i32, _c_float_p, sz],
        "lenia_read_state": [vp, i32, _c_float_p, sz],
        "lenia_write_state_device": [vp, i32, vp, sz],
        "lenia_read_state_device": [vp, i32, vp, sz],
        "lenia_write_states": [vp, _c_float_p, sz],
        "lenia_write_states_async": [vp, _c_float_p, sz],
        "lenia_read_states": [vp, _c_float_p, sz],
        "lenia_read_states_async": [vp, _c_float_p, sz],
        "lenia_step": [vp, u32],
        "lenia_step_timed": [vp, u32, _c_float_p],
        "lenia_sync": [vp],
        "lenia_tick": [vp, ctypes.POINTER(ctypes.c_uint64)],
        "lenia_seed_tiles": [vp, i32, u32, _c_float_p, i32, i32, i32],
        "lenia_seed_patches": [vp, i32, u32, ctypes.POINTER(ctypes.c_int32), i32],
        "lenia_cells_per_step": [vp, ctypes.POINTER(ctypes.c_uint64)],
        "lenia_memory_bytes": [vp, ctypes.POINTER(ctypes.c_uint64)],
        "lenia_read_field_u": [vp, i32, i32, _c_float_p, sz],
        "lenia_read_spectrum": [vp, i32, i32, _c_float_p, sz],
        "lenia_world_stats": [vp, _c_float_p, sz],
        "lenia_autotune": [vp],
        "lenia_set_variants": [vp, i32, i32],
        "lenia_class_variants": [vp, ctypes.POINTER(ctypes.c_int32), sz, ctypes.POINTER(ctypes.c_size_t)],
        "lenia_class_shapes": [vp, ctypes.POINTER(ctypes.c_int32), sz, ctypes.POINTER(ctypes.c_size_t)],
        "lenia_set_chunk_budget": [vp, u32],
        "lenia_set_chunk_lanes": [vp, i32],
        "lenia_set_resident": [vp, i32],
        "lenia_set_persistent": [vp, i32],
        "lenia_set_tc_rows": [vp, i32],
        "lenia_set_tc_variant": [vp, i32],
        "lenia_set_branch_split": [vp, ctypes.c_int64, i32],
        "lenia_branch_split": [vp, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int32)],
        "lenia_profile_step": [vp, u32, _c_float_p],
        "lenia_profile_classes": [vp, u32, _c_float_p, sz, ctypes.POINTER(ctypes.c_size_t)],
        "lenia_kernel_spectrum": [ctypes.POINTER(LeniaKernel), u32, u32, _c_float_p, sz],
        "lenia_tc_selftest": [i32, i32, i32, _c_float_p, _c_float_p, _c_float_p],
        "lenia_tc_set_wait_limit": [vp, i32],
        "lenia_persist_set_wait_limit": [vp, i32],
        "lenia_step_noalloc": [vp, u32, u32, vp, ctypes.c_float, ctypes.c_float, ctypes.c_float, u32, vp],
        "lenia_seed_rule": [vp, i32, u32, i32],
        "lenia_render": [vp, i32, i32, ctypes.c_float, ctypes.c_float, ctypes.c_float, u32, u32, u32, i32, vp],
        "lenia_mlp_create": [u32, u32, ctypes.POINTER(vp)],
        "lenia_mlp_destroy": [vp],
        "lenia_mlp_param_count": [ctypes.POINTER(u32)],
        "lenia_mlp_set_params": [vp, _c_float_p, sz],
        "lenia_mlp_get_params": [vp, _c_float_p, sz],
        "lenia_mlp_gradients": [vp, _c_float_p, _c_float_p, u32, _c_float_p, _c_float_p],
        "lenia_mlp_train_step": [vp, _c_float_p, _c_float_p, u32, ctypes.c_float, _c_float_p],
        "lenia_mlp_predict": [vp, _c_float_p, u32, _c_float_p],
    }
    for name, args in sig.items():
        f = getattr(L, name)
        f.restype = ctypes.c_int
        f.argtypes = args


def load():
    """Load the engine library (no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("liblenia_gb300.so is not built; run auto_gb300.native.build() "
                              "(or __graft_entry__.build())")
        L = ctypes.CDLL(LIB_PATH)
        _declare(L)
        _lib = L
    return _lib


def check(rc, ctx=None):
    if rc != 0:
        msg = load().lenia_last_error(ctx)
        raise LeniaError(rc, msg.decode() if msg else "error")
    return rc


def fptr(a):
    return a.ctypes.data_as(_c_float_p)
