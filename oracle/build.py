"""Build recipe for the CPU oracle (test infrastructure, not part of the shipped library).

Compiles oracle/lenia_oracle.c into oracle/_build/liblenia_oracle.so with gcc.  The reference
project itself (Rust + WGSL on wgpu/Vulkan) cannot be built in this image: there is no Rust
toolchain and no graphics stack, so the oracle is a C restatement of its f32 pass sequence.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liblenia_oracle.so")
SRC = os.path.join(HERE, "lenia_oracle.c")


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O2", "-std=c11", "-ffp-contract=off", "-fPIC", "-shared", "-pthread",
           SRC, "-o", tmp, "-lm"]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
