"""Build the in-tree CUDA library fsibe_2d_gb300/_lib/libfsibe_gb300.so for sm_103a.

Every .cu under csrc/ is compiled by its own nvcc process (in parallel), then linked into one
shared library exporting the C ABI of include/fsibe.h.  Usage:  python -m fsibe_2d_gb300.build
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
BUILD_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libfsibe_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
          "--expt-relaxed-constexpr", "-Wno-deprecated-gpu-targets"]
# per-file extra flags: the solid side keeps multiply and add separate (no FMA contraction)
EXTRA = {"solid.cu": ["-fmad=false"]}


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return exe


def _compile(src, verbose=False):
    base = os.path.basename(src)
    obj = os.path.join(BUILD_DIR, base + ".o")
    deps = [src] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cuh")]
    deps.append(os.path.join(os.path.dirname(HERE), "include", "fsibe.h"))
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in deps):
        return obj, ""
    cmd = [nvcc()] + ARCH + COMMON + EXTRA.get(base, []) + ["-c", src, "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError(f"nvcc failed for {base}:\n{p.stderr}")
    return obj, p.stderr


def build(verbose=False, jobs=None):
    os.makedirs(OUT_DIR, exist_ok=True)
    os.makedirs(BUILD_DIR, exist_ok=True)
    srcs = sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))
    jobs = jobs or max(1, min(len(srcs), os.cpu_count() or 4))
    objs = []
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        for obj, log in ex.map(lambda s: _compile(s, verbose), srcs):
            objs.append(obj)
            if verbose and log:
                sys.stderr.write(log)
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        subprocess.check_call(cmd)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
