"""Build recipe of the product: libgpuropolis.so (CUDA kernels + C ABI + host
library) and the `gpuropolis` command-line tool, for sm_103a only.

Each translation unit compiles in its own nvcc/g++ process, in parallel, and
is rebuilt only when a source or header is newer than its object.  Outputs go
to gpuropolis_gb300/_lib/ (git-ignored).
"""
import concurrent.futures as cf
import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
ROOT = os.path.dirname(HERE)
INC = os.path.join(ROOT, "include")
LIB_DIR = os.path.join(HERE, "_lib")
OBJ_DIR = os.path.join(LIB_DIR, "obj")
LIB = os.path.join(LIB_DIR, "libgpuropolis.so")
CLI = os.path.join(LIB_DIR, "gpuropolis")

NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler",
              "-ffp-contract=off", "-I", INC, "-I", CSRC]
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function",
             "-I", INC, "-I", CSRC, "-I", "/usr/local/cuda/include"]


def _headers():
    return glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(INC, "*.h"))


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n%s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def build(verbose=False, jobs=None):
    os.makedirs(OBJ_DIR, exist_ok=True)
    hdrs = _headers()
    cu = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    cpp = sorted(p for p in glob.glob(os.path.join(CSRC, "*.cpp")) if not p.endswith("gpr_cli.cpp"))
    steps = []
    objs = []
    for src in cu:
        obj = os.path.join(OBJ_DIR, os.path.basename(src) + ".o")
        objs.append(obj)
        if _stale(obj, [src] + hdrs):
            steps.append([NVCC] + ARCH + NVCC_FLAGS + ["-c", src, "-o", obj])
    for src in cpp:
        obj = os.path.join(OBJ_DIR, os.path.basename(src) + ".o")
        objs.append(obj)
        if _stale(obj, [src] + hdrs):
            steps.append(["g++"] + CXX_FLAGS + ["-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=jobs or max(2, os.cpu_count() or 2)) as ex:
        for out in ex.map(_run, steps):
            if verbose and out.strip():
                print(out)
    if _stale(LIB, objs):
        _run([NVCC] + ARCH + ["-shared", "-o", LIB + ".tmp"] + objs + ["-lcudart"])
        os.replace(LIB + ".tmp", LIB)
    cli_src = os.path.join(CSRC, "gpr_cli.cpp")
    if os.path.exists(cli_src) and _stale(CLI, [cli_src, LIB] + hdrs):
        _run(["g++"] + CXX_FLAGS + ["-o", CLI + ".tmp", cli_src, "-L", LIB_DIR, "-lgpuropolis",
                                    "-Wl,-rpath,$ORIGIN"])
        os.replace(CLI + ".tmp", CLI)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
