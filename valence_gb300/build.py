"""Build recipe for the sm_103a library (libvsvb_gb300.so), in-tree.

Each CUDA translation unit is compiled in parallel with
    nvcc -O3 -gencode arch=compute_103a,code=sm_103a -lineinfo
and linked into valence_gb300/_build/libvsvb_gb300.so (CUDA runtime linked
statically).  No torch types cross the library boundary.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libvsvb_gb300.so")
CU = ["eri.cu", "eri_f64.cu", "eri_f32.cu", "eri_df64.cu", "density.cu", "onee.cu", "handle.cu", "peak.cu",
      "detfactor.cu", "optimize.cu", "block.cu", "core.cu"]
CPP = ["input.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _stale(obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False):
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    headers = [os.path.join(SRC, f) for f in os.listdir(SRC) if f.endswith((".h", ".cuh", ".inc"))]
    headers.append(os.path.join(os.path.dirname(HERE), "include", "vsvb_gpu.h"))
    jobs = []
    for f in CU:
        src, obj = os.path.join(SRC, f), os.path.join(OUT, f.replace(".cu", ".o"))
        if force or _stale(obj, [src] + headers):
            jobs.append([nvcc, "-O3", "-std=c++17", "-Xcompiler", "-fPIC", *ARCH, "-lineinfo", "-c", src, "-o", obj])
    for f in CPP:
        src, obj = os.path.join(SRC, f), os.path.join(OUT, f.replace(".cpp", ".o"))
        if force or _stale(obj, [src] + headers):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-c", src, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("compile failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        return cmd[-1]

    with cf.ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
        for o in ex.map(run, jobs):
            if verbose:
                print("built", o, file=sys.stderr)
    objs = [os.path.join(OUT, f.rsplit(".", 1)[0] + ".o") for f in CU + CPP]
    if force or jobs or _stale(LIB, objs):
        run([nvcc, "-shared", *ARCH, "-o", LIB, *objs])
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
