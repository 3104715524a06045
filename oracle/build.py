"""Build recipe for the CPU oracle (test infrastructure only).

Compiles pt_oracle.c into oracle/libpt_oracle.so with FP contraction off so
that its FP32 arithmetic follows the written operation order exactly.  The
reference's own sources cannot be compiled here (its CUDA uses texture
references and cudaThreadSynchronize, both removed in CUDA 13, and its host
code needs Qt5/OpenEXR/GLEW), so there is no oracle/_ref build.
"""
import os
import platform
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "pt_oracle.c")
OUT = os.path.join(HERE, "libpt_oracle.so")


def build(force=False, verbose=False):
    if (not force and os.path.exists(OUT)
            and os.path.getmtime(OUT) >= os.path.getmtime(SRC)
            and os.path.getmtime(OUT) >= os.path.getmtime(
                os.path.join(HERE, "..", "include", "painttween.h"))):
        return OUT
    flags = ["-O2", "-std=gnu11", "-fPIC", "-shared", "-ffp-contract=off",
             "-fno-fast-math", "-fopenmp", "-Wall", "-Wno-unused-function"]
    if platform.machine() in ("x86_64", "AMD64"):
        flags.append("-mfma")  # fmaf() as one instruction; results unchanged
    cmd = ["gcc"] + flags + [SRC, "-o", OUT + ".tmp", "-lm"]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    os.replace(OUT + ".tmp", OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
