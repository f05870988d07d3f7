"""auto_gb300: a Lenia-family FFT stepping engine for one NVIDIA GB300 (sm_103a).

The compute path is hand-written CUDA in auto_gb300/csrc behind the C ABI of
include/lenia_gb300.h; this package is the Python host side: the world/automaton registry
(program.py, mirroring the reference's automata::Entry / Program) and the Sim wrapper
(sim.py, mirroring the reference's Sim).
"""
from . import configs
from ._lib import (PATH_BF16X3, PATH_FP32, PATH_RADIX2, PATH_TF32, RULE_LENIA, RULE_MNCA, RULE_SMOOTHLIFE,
                   SHAPE_LENIA, SHAPE_RING, SHAPE_SL_INNER, SHAPE_SL_OUTER, LeniaError)
from .program import ALL, Entry, Kernel, Seed, World, build, find, fit_size, lenia, mnca, mnca_shaped, smoothlife
from .sim import Sim

__all__ = ["Sim", "World", "Kernel", "Seed", "Entry", "ALL", "build", "find", "fit_size", "lenia", "smoothlife",
           "mnca", "mnca_shaped", "configs", "LeniaError", "PATH_FP32", "PATH_TF32", "PATH_BF16X3", "PATH_RADIX2",
           "RULE_LENIA", "RULE_SMOOTHLIFE", "RULE_MNCA", "SHAPE_LENIA", "SHAPE_SL_INNER", "SHAPE_SL_OUTER",
           "SHAPE_RING"]
