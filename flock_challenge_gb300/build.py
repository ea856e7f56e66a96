"""Builds the CUDA library libflock_gpu.so in-tree for sm_103a.

Each translation unit under csrc/ is compiled by nvcc in parallel and linked
with -shared; outputs go to flock_challenge_gb300/_build/ (git-ignored).
Rebuilds only when a source or header is newer than the library.
"""
import concurrent.futures as cf
import glob
import os
import platform
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(BUILD, "libflock_gpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# On an Arm host the host-side GF(2^128) products use PMULL (the crypto
# extension of every Grace core); other hosts keep the portable product.
HOST_ARCH = ["-Xcompiler", "-march=armv8-a+crypto"] if platform.machine() == "aarch64" else []


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libflock_gpu.so")
    return exe


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))


def _deps():
    return _sources() + glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + \
        glob.glob(os.path.join(ROOT, "include", "*.h")) + [os.path.abspath(__file__)]


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(d) <= t for d in _deps())


def build(verbose=False, extra_flags=()):
    if up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    exe = nvcc()
    flags = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", os.path.join(ROOT, "include"),
             *ARCH, *HOST_ARCH, *extra_flags]

    def compile_one(src):
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        cmd = [exe, *flags, "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, _sources()))
    tmp = LIB + ".tmp"
    r = subprocess.run([exe, "-shared", *ARCH, "-o", tmp, *objs, "-lcudart"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(verbose="-v" in sys.argv))
