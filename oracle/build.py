"""Build recipe for the CPU oracle (test infrastructure only).

Compiles pt_oracle.c into oracle/libpt_oracle.so with FP contraction off so
that its FP32 arithmetic follows the written operation order exactly.

The reference's kernels and drivers cannot be compiled here (its CUDA uses
texture references and cudaThreadSynchronize, both removed in CUDA 13, and
its host code needs Qt5/OpenEXR/GLEW).  Its device helper header
(texSynth_util.h: colour conversion, exemplar basis and coordinates,
clamping, squared differences, ribbon unpacking) and its host pyramid code
(downsample.cpp, given the small QtCore container shim in qt_shim/) do
compile for the host: where the reference tree is present, build_ref()
compiles them through ref_helpers.cpp and ref_downsample.cpp into
oracle/_ref/libref_helpers.so, and the helper header through
ref_helpers_dev.cu into an sm_103a cubin, against which the tests check the
oracle's restatements.
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


def _reference_src():
    """The reference's src/PaintTweenCUDA: $PT_REFERENCE_SRC, else a
    `reference` tree beside this repository."""
    env = os.environ.get("PT_REFERENCE_SRC")
    if env:
        return env
    return os.path.normpath(os.path.join(HERE, "..", "..", "reference", "src", "PaintTweenCUDA"))


REF_SRC = _reference_src()
REF_SHIM = os.path.join(HERE, "ref_helpers.cpp")
REF_DOWNSAMPLE_SHIM = os.path.join(HERE, "ref_downsample.cpp")
QT_SHIM = os.path.join(HERE, "qt_shim")
REF_OUT = os.path.join(HERE, "_ref", "libref_helpers.so")


def build_ref(force=False, verbose=False):
    """oracle/_ref/libref_helpers.so from the reference's texSynth_util.h and
    downsample.cpp (over the QtCore container shim in oracle/qt_shim), or
    None when the reference tree is not present."""
    header = os.path.join(REF_SRC, "texSynth_util.h")
    if not os.path.exists(header):
        return None
    deps = [REF_SHIM, REF_DOWNSAMPLE_SHIM, os.path.join(QT_SHIM, "QtCore", "qt_shim_core.h")]
    if (not force and os.path.exists(REF_OUT)
            and all(os.path.getmtime(REF_OUT) >= os.path.getmtime(d) for d in deps)):
        build_ref_cubin(verbose=verbose)
        build_ref_gauss(verbose=verbose)
        return REF_OUT
    cuda_inc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
    os.makedirs(os.path.dirname(REF_OUT), exist_ok=True)
    # contraction on, as nvcc compiles the reference's device code (--fmad=true)
    flags = ["-O2", "-std=c++14", "-fPIC", "-shared", "-w", "-ffp-contract=fast"]
    if platform.machine() in ("x86_64", "AMD64"):
        flags.append("-mfma")
    cmd = ["g++"] + flags + ["-I", QT_SHIM, "-I", os.path.join(QT_SHIM, "QtCore"), "-I", REF_SRC, "-I", cuda_inc, REF_SHIM, REF_DOWNSAMPLE_SHIM,
                             os.path.join(REF_SRC, "downsample.cpp"), "-o", REF_OUT + ".tmp", "-lm"]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    os.replace(REF_OUT + ".tmp", REF_OUT)
    build_ref_cubin(force=force, verbose=verbose)
    build_ref_gauss(force=force, verbose=verbose)
    return REF_OUT


REF_GAUSS_SHIM = os.path.join(HERE, "ref_gauss.cu")
REF_GAUSS_OUT = os.path.join(HERE, "_ref", "libref_gauss.so")


def build_ref_gauss(force=False, verbose=False):
    """oracle/_ref/libref_gauss.so: the reference's allocateGaussianKernel
    (convolution.cu) compiled for the host by nvcc over the QtCore container
    shim, or None without the reference tree."""
    if not os.path.exists(os.path.join(REF_SRC, "convolution.cu")):
        return None
    if (not force and os.path.exists(REF_GAUSS_OUT)
            and os.path.getmtime(REF_GAUSS_OUT) >= os.path.getmtime(REF_GAUSS_SHIM)):
        return REF_GAUSS_OUT
    nvcc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    os.makedirs(os.path.dirname(REF_GAUSS_OUT), exist_ok=True)
    cmd = [nvcc, "-shared", "-Xcompiler", "-fPIC", "-gencode", "arch=compute_103a,code=sm_103a", "-w",
           "-I", QT_SHIM, "-I", os.path.join(QT_SHIM, "QtCore"), "-I", REF_SRC, REF_GAUSS_SHIM,
           "-o", REF_GAUSS_OUT + ".tmp"]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    os.replace(REF_GAUSS_OUT + ".tmp", REF_GAUSS_OUT)
    return REF_GAUSS_OUT


REF_DEV_SHIM = os.path.join(HERE, "ref_helpers_dev.cu")
REF_CUBIN = os.path.join(HERE, "_ref", "ref_helpers.cubin")


def build_ref_cubin(force=False, verbose=False):
    """oracle/_ref/ref_helpers.cubin: texSynth_util.h compiled by nvcc for
    sm_103a with nvcc's default arithmetic, or None without the reference
    tree.  A cubin is loaded by the driver, so one built here runs on any
    host with a GB300."""
    if not os.path.exists(os.path.join(REF_SRC, "texSynth_util.h")):
        return None
    if (not force and os.path.exists(REF_CUBIN)
            and os.path.getmtime(REF_CUBIN) >= os.path.getmtime(REF_DEV_SHIM)):
        return REF_CUBIN
    nvcc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    os.makedirs(os.path.dirname(REF_CUBIN), exist_ok=True)
    cmd = [nvcc, "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-w", "-I", REF_SRC,
           REF_DEV_SHIM, "-o", REF_CUBIN + ".tmp"]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    os.replace(REF_CUBIN + ".tmp", REF_CUBIN)
    return REF_CUBIN


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
    print(build_ref(force="--force" in sys.argv, verbose=True))
