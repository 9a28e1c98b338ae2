"""Build libtvgb.so (the CUDA kernels and their C ABI) in-tree.

Every translation unit in csrc/ is compiled for sm_103a only
(-gencode arch=compute_103a,code=sm_103a) in parallel, then linked into
tiralib_gb300/_build/libtvgb.so.  No CMake, no torch extension machinery.
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libtvgb.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc_path():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _flags():
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
                   "-Xcompiler", "-fPIC", "-Xcompiler", "-O2", "-I", os.path.join(HERE, "..", "include")]


def build(verbose=False, extra=(), out_dir=None):
    out_dir = out_dir or OUT_DIR
    os.makedirs(out_dir, exist_ok=True)
    nvcc = nvcc_path()
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    objs = []

    def compile_one(src):
        obj = os.path.join(out_dir, os.path.basename(src)[:-3] + ".o")
        cmd = [nvcc, "-c", src, "-o", obj] + _flags() + list(extra)
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr.strip():
            print(r.stderr, flush=True)
        return obj

    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 4))) as ex:
        objs = list(ex.map(compile_one, srcs))
    lib = os.path.join(out_dir, "libtvgb.so")
    tmp = lib + ".tmp"
    cmd = [nvcc, "-shared", "-o", tmp] + objs + ARCH + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    args = sys.argv[1:]
    out = None
    if len(args) >= 2 and args[0] == "--out":
        out, args = args[1], args[2:]
    print(build(verbose=True, extra=args, out_dir=out))
