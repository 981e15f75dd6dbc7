"""Build recipe for libcans_gb300.so (the C-ABI library, sm_103a only).

nvcc compiles each translation unit in parallel and links one shared library
in-tree at cans_gb300/_build/libcans_gb300.so.  No torch extension is involved:
the library exposes plain `extern "C"` entry points (include/cans_gb300.h).
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC_DIR = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libcans_gb300.so")
SOURCES = ["solver.cu", "stencil.cu", "stencil32.cu", "refine.cu", "batch.cu", "boxes.cu", "adjoint.cu", "io.cu", "stats.cu", "initflow.cu", "ztile.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
         "-I" + os.path.join(ROOT, "include")]


def _nvcc():
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def _deps():
    files = [os.path.join(SRC_DIR, f) for f in os.listdir(SRC_DIR)]
    files.append(os.path.join(ROOT, "include", "cans_gb300.h"))
    return max(os.path.getmtime(f) for f in files)


def build(force=False, verbose=False, extra=()):
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _deps():
        return LIB
    nvcc = _nvcc()

    def compile_one(src):
        obj = os.path.join(OUT_DIR, os.path.splitext(src)[0] + ".o")
        cmd = [nvcc, *ARCH, *FLAGS, *extra, "-c", os.path.join(SRC_DIR, src), "-o", obj]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr}")
        return obj, r.stderr

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(compile_one, SOURCES))
    if verbose:
        for _, log in results:
            sys.stderr.write(log)
    tmp = LIB + ".tmp"
    subprocess.run([nvcc, *ARCH, "-shared", "-o", tmp, *[o for o, _ in results], "-lcudart"], check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
