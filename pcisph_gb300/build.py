"""Build the CUDA library in-tree: pcisph_gb300/libpcisph_gb300.so (sm_103a only).

Each translation unit is compiled by nvcc in parallel, then linked into one
shared library whose exported symbols are exactly the C ABI of
include/pcisph_gpu.h. No torch types cross that boundary.
"""
import concurrent.futures
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libpcisph_gb300.so")
SOURCES = ["context.cu", "batch.cu", "step_kernels.cu", "sweep_kernels.cu", "list_kernels.cu", "spatial_order.cu", "render.cu", "radix_sort.cu",
           "radix_sort_noalloc.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2,-fvisibility=hidden",
              "-I", os.path.join(ROOT, "include")]


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build pcisph_gb300")
    return exe


def _deps():
    out = [os.path.join(ROOT, "include", "pcisph_gpu.h")]
    for f in os.listdir(CSRC):
        out.append(os.path.join(CSRC, f))
    return out


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False):
    """Compile and link the library if any source changed; returns its path."""
    deps = _deps()
    if not force and not _stale(LIB, deps):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    exe = nvcc()

    def compile_one(src):
        obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
        cmd = [exe, *ARCH, *NVCC_FLAGS, "-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr)
        return obj

    with concurrent.futures.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + ".tmp"
    r = subprocess.run([exe, *ARCH, "-shared", "-o", tmp, *objs], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


CLI_SRC = os.path.join(PKG, "cli", "pcisph_run.cpp")
CLI = os.path.join(PKG, "pcisph_run")


def build_cli(force=False):
    """The headless C++ runner (cli/pcisph_run.cpp) against the library; returns its path."""
    lib = build()
    deps = [CLI_SRC, lib, os.path.join(ROOT, "include", "pcisph_fluid.hpp"), os.path.join(ROOT, "include", "pcisph_gpu.h")]
    if not force and not _stale(CLI, deps):
        return CLI
    cxx = shutil.which("g++") or "g++"
    cmd = [cxx, "-std=c++17", "-O2", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"), CLI_SRC, "-o", CLI + ".tmp", "-L", PKG,
           "-l:libpcisph_gb300.so", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"g++ failed on the runner:\n{r.stdout}\n{r.stderr}")
    os.replace(CLI + ".tmp", CLI)
    return CLI


if __name__ == "__main__":
    print(build(force=True, verbose=True))
