"""Build recipe of the reference-kernel port (test and baseline
infrastructure only; nothing in the product links it).

The reference's CUDA code (src/PaintTweenCUDA/texSynth_kernel.cu,
convolution.cu, advectedBuffers.cpp and the headers they include) is
compiled unchanged, with three things supplied from this directory:
  - cudaImagePyramid.h: the reference's pyramid macros over texture objects
    (its texture references were removed in CUDA 13);
  - refport_compat.h, force-included: cudaThreadSynchronize, also removed in
    CUDA 13, as cudaDeviceSynchronize;
  - refport_pyramid.cu and refport_replay.cu: the pyramid host class and a C
    driver with the oracle's step surface (the Qt/OpenEXR host code around
    the kernels is not built);
and the QtCore container shim of oracle/qt_shim.

stage() copies the reference files into oracle/_ref/refport_src/ where the
reference tree is present (this directory is git-ignored; it travels with the
working copy to a GPU host, where build() compiles the host side for that
machine).  build() writes oracle/_ref/libref_texsynth.so.  Compiler flags are
those of the reference's CMake build (no fast-math; nvcc's default
multiply-add contraction) for sm_103a.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
ROOT = os.path.dirname(ORACLE)
STAGE = os.path.join(ORACLE, "_ref", "refport_src")
OUT = os.path.join(ORACLE, "_ref", "libref_texsynth.so")
BUILD = os.path.join(ORACLE, "_ref", "refport_build")
QT_SHIM = os.path.join(ORACLE, "qt_shim")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"

# the reference files the port compiles (cudaImagePyramid.h is replaced)
REF_FILES = ["texSynth_kernel.cu", "texSynth_kernel.h", "texSynth_util.h", "texSynth_interface.h", "types.h",
             "cutil_math.h", "cudaImageBuffer.h", "cudaHostUtil.h", "cudaTexture.h", "convolution.cu",
             "convolution.h", "workingBuffers.h", "advectedBuffers.h", "advectedBuffers.cpp", "imagePyramid.h",
             "downsample.h"]
SHIMS = ["cudaImagePyramid.h", "refport_compat.h", "refport_pyramid.cu", "refport_replay.cu"]


def stage(src=None):
    """Copies the reference files into oracle/_ref/refport_src; returns the
    directory, or None when neither the reference tree nor a staged copy
    exists."""
    from oracle import build as ob
    src = src or ob.REF_SRC
    if not os.path.exists(os.path.join(src, "texSynth_kernel.cu")):
        return STAGE if staged() else None
    os.makedirs(STAGE, exist_ok=True)
    for f in REF_FILES:
        s, d = os.path.join(src, f), os.path.join(STAGE, f)
        if not os.path.exists(d) or os.path.getmtime(d) < os.path.getmtime(s):
            shutil.copy2(s, d)
    return STAGE


def staged():
    return all(os.path.exists(os.path.join(STAGE, f)) for f in REF_FILES)


def _cuda_home():
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and os.path.exists(os.path.join(cand, "bin", "nvcc")):
            return cand
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found")


def build(force=False, verbose=False):
    """oracle/_ref/libref_texsynth.so, or None when the port's sources are not
    staged."""
    if stage() is None:
        return None
    deps = [os.path.join(STAGE, f) for f in REF_FILES] + [os.path.join(HERE, f) for f in SHIMS] + [
        os.path.join(QT_SHIM, "QtCore", "qt_shim_core.h"), os.path.join(ROOT, "include", "painttween.h")]
    if not force and os.path.exists(OUT) and os.path.getmtime(OUT) >= max(os.path.getmtime(d) for d in deps):
        return OUT
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(BUILD, exist_ok=True)
    inc = ["-I" + HERE, "-I" + STAGE, "-I" + QT_SHIM, "-I" + os.path.join(QT_SHIM, "QtCore"),
           "-I" + os.path.join(ROOT, "include")]
    cu = [os.path.join(STAGE, "texSynth_kernel.cu"), os.path.join(STAGE, "convolution.cu"),
          os.path.join(HERE, "refport_pyramid.cu"), os.path.join(HERE, "refport_replay.cu")]
    jobs, objs = [], []
    for f in cu:
        o = os.path.join(BUILD, os.path.basename(f) + ".o")
        objs.append(o)
        jobs.append([nvcc, ARCH, "-O2", "-std=c++14", "-w", "-Xcompiler", "-fPIC", "-include",
                     os.path.join(HERE, "refport_compat.h")] + inc + ["-c", f, "-o", o])
    o = os.path.join(BUILD, "advectedBuffers.o")
    objs.append(o)
    jobs.append(["g++", "-O2", "-std=c++14", "-w", "-fPIC", "-include", os.path.join(HERE, "refport_compat.h"),
                 "-I" + os.path.join(cuda, "include")] + inc + ["-c", os.path.join(STAGE, "advectedBuffers.cpp"),
                                                              "-o", o])
    procs = []
    for cmd in jobs:
        if verbose:
            print(" ".join(cmd))
        procs.append(subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT))
    failed = []
    for cmd, p in zip(jobs, procs):
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append(" ".join(cmd[-3:]) + "\n" + out.decode(errors="replace"))
    if failed:
        raise RuntimeError("reference port build failed:\n" + "\n".join(failed))
    link = [nvcc, ARCH, "-shared", "-o", OUT + ".tmp"] + objs + ["-lcudart_static", "-lrt", "-lpthread", "-ldl"]
    if verbose:
        print(" ".join(link))
    subprocess.check_call(link)
    os.replace(OUT + ".tmp", OUT)
    return OUT


if __name__ == "__main__":
    sys.path.insert(0, ROOT)
    print(build(force="--force" in sys.argv, verbose=True))
