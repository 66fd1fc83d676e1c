"""In-tree build of the CUDA library (libvecgeom_gb300.so) for sm_103a.

Host sources (*.cpp) are compiled with g++ and device sources (*.cu) with nvcc, in
parallel; nothing goes outside vecgeom_gb300/_build and vecgeom_gb300/_lib.

Floating-point flags are part of the parity contract: device code is compiled with
--fmad=false and IEEE division and square root, host code with -ffp-contract=off, so the
plain-FP64 path rounds every operation exactly as the reference's scalar FP64 build does.
The mixed-precision kernels request fused multiply-adds explicitly (fmaf) where they want them.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIBDIR, "libvecgeom_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return cand


def _cuda_include():
    nv = _nvcc()
    root = os.path.dirname(os.path.dirname(os.path.realpath(nv)))
    return os.path.join(root, "include")


def _commands():
    nvcc = _nvcc()
    inc = ["-I", CSRC, "-I", os.path.join(HERE, "..", "include")]
    host_flags = ["-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-Wall",
                  "-I", _cuda_include(), *inc]
    dev_flags = [*ARCH, "-lineinfo", "-O3", "-std=c++17", "--fmad=false", "-prec-div=true", "-prec-sqrt=true",
                 "-ftz=false", "-Xcompiler", "-fPIC,-ffp-contract=off", "-Xptxas", "-warn-spills", *inc]
    cmds = []
    for f in sorted(os.listdir(CSRC)):
        src = os.path.join(CSRC, f)
        if f.endswith(".cpp"):
            obj = os.path.join(BUILD, f[:-4] + ".o")
            cmds.append((src, obj, ["g++", *host_flags, "-c", src, "-o", obj]))
        elif f.endswith(".cu"):
            obj = os.path.join(BUILD, f[:-3] + ".o")
            cmds.append((src, obj, [nvcc, *dev_flags, "-c", src, "-o", obj]))
    return cmds


def build(force=False, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(HERE, "..", "include", "vecgeom_gb300.h"))
    newest_hdr = max(os.path.getmtime(h) for h in headers)
    todo = []
    objs = []
    for src, obj, cmd in _commands():
        objs.append(obj)
        if force or not os.path.exists(obj) or os.path.getmtime(obj) < max(os.path.getmtime(src), newest_hdr):
            todo.append(cmd)

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr, flush=True)

    with ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 4)) as ex:
        list(ex.map(run, todo))
    if todo or not os.path.exists(LIB):
        run([_nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lpthread"])
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
