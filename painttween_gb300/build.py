"""In-tree build of libpainttween_gb300.so for sm_103a.

Translation units compiled in parallel: the kernels with nvcc
(-fmad=false: multiply-adds are fused only where the source writes fmaf) and
the host code with g++ against the CUDA runtime; linked with nvcc (static
cudart).  No CPU fallback is built.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libpainttween_gb300.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def _cuda_home():
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and os.path.exists(os.path.join(cand, "bin", "nvcc")):
            return cand
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build painttween_gb300")


def _sources():
    return [os.path.join(CSRC, f) for f in sorted(os.listdir(CSRC))] + [
        os.path.join(ROOT, "include", "painttween.h")]


def build(force=False, verbose=False):
    srcs = _sources()
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(s) for s in srcs)):
        return LIB
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(BUILD, exist_ok=True)
    inc = ["-I" + os.path.join(ROOT, "include"), "-I" + CSRC]
    cu_files = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    objs = [os.path.join(BUILD, f[:-3] + ".o") for f in cu_files]
    cpp_files = sorted(f for f in os.listdir(CSRC) if f.endswith(".cpp"))
    h_objs = [os.path.join(BUILD, f[:-4] + ".o") for f in cpp_files]
    jobs = [[nvcc, ARCH, "-lineinfo", "-O3", "-fmad=false", "-std=c++17", "-Xcompiler", "-fPIC",
             "--expt-relaxed-constexpr"] + inc + ["-c", os.path.join(CSRC, f), "-o", o]
            for f, o in zip(cu_files, objs)]
    for f, o in zip(cpp_files, h_objs):
        jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-Wall", "-Wno-unused-function",
                     "-I" + os.path.join(cuda, "include")] + inc + ["-c", os.path.join(CSRC, f), "-o", o])
    procs = []
    for cmd in jobs:
        if verbose:
            print(" ".join(cmd))
        procs.append(subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT))
    failed = []
    for cmd, p in zip(jobs, procs):
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append(out.decode(errors="replace"))
        elif verbose and out:
            print(out.decode(errors="replace"))
    if failed:
        raise RuntimeError("painttween_gb300 build failed:\n" + "\n".join(failed))
    link = [nvcc, ARCH, "-shared", "-o", LIB + ".tmp"] + objs + h_objs + ["-lcudart_static", "-lrt", "-lpthread",
                                                                     "-ldl"]
    if verbose:
        print(" ".join(link))
    subprocess.check_call(link)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
