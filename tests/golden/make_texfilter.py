"""Writes tests/golden/texfilter_gb300.npz: bilinear texture fetches recorded
on a GB300, the fixture against which tests/test_oracle.py checks the
oracle's emulation of the texture unit (PT_FILTER_TEXTURE).

Run on a machine with the GPU:  python tests/golden/make_texfilter.py
It builds texfilter_probe.cu with nvcc for sm_103a, runs it into a temporary
directory and stores every case (texels, coordinates, fetched values).
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def read_case(path):
    b = open(path, "rb").read()
    W, H, L, C, n = np.frombuffer(b[:20], np.int32)
    off = 20
    tex = np.frombuffer(b[off:off + W * H * L * C * 4], np.float32).reshape(L, H, W, C)
    off += W * H * L * C * 4
    q = np.frombuffer(b[off:off + 3 * n * 4], np.float32).reshape(n, 3)
    off += 3 * n * 4
    out = np.frombuffer(b[off:off + C * n * 4], np.float32).reshape(n, C)
    return tex, q, out


def main():
    nvcc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    with tempfile.TemporaryDirectory() as tmp:
        exe = os.path.join(tmp, "texfilter_probe")
        subprocess.check_call([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O2",
                               os.path.join(HERE, "texfilter_probe.cu"), "-o", exe])
        subprocess.check_call([exe, tmp])
        cases = {}
        for f in sorted(os.listdir(tmp)):
            if f.endswith(".bin"):
                tex, q, out = read_case(os.path.join(tmp, f))
                name = f[:-4]
                cases[name + "/tex"] = tex
                cases[name + "/q"] = q
                cases[name + "/out"] = out
        gpu = subprocess.run(["nvidia-smi", "--query-gpu=name,driver_version", "--format=csv,noheader"],
                             capture_output=True, text=True).stdout.strip()
        cases["meta/gpu"] = np.array(gpu)
        np.savez_compressed(os.path.join(HERE, "texfilter_gb300.npz"), **cases)
        print("wrote texfilter_gb300.npz:", ", ".join(sorted({k.split("/")[0] for k in cases})))


if __name__ == "__main__":
    sys.exit(main())
