"""Build the oracle shared library (test infrastructure; see ref_base.h).

g++ -O2 -std=c++17 -ffp-contract=off: no floating-point contraction, so each +, -, *, /
and sqrt rounds exactly as the reference's scalar FP64 build does on x86-64; aarch64 gcc
would otherwise fuse multiply-adds by default.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")
SOURCES = sorted(f for f in os.listdir(HERE) if f.endswith(".cpp"))
FLAGS = ["-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-Wall", "-Wno-unused-function"]


def build(force=False, verbose=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    headers = [os.path.join(HERE, f) for f in os.listdir(HERE) if f.endswith(".h")]
    newest_hdr = max(os.path.getmtime(h) for h in headers)
    objs = []
    jobs = []
    for src in SOURCES:
        sp = os.path.join(HERE, src)
        obj = os.path.join(OUT_DIR, src[:-4] + ".o")
        objs.append(obj)
        if force or not os.path.exists(obj) or os.path.getmtime(obj) < max(os.path.getmtime(sp), newest_hdr):
            jobs.append(["g++", *FLAGS, "-c", sp, "-o", obj])

    def run(cmd):
        if verbose:
            print(" ".join(cmd))
        subprocess.run(cmd, check=True)

    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        list(ex.map(run, jobs))
    if jobs or not os.path.exists(LIB):
        run(["g++", "-shared", "-o", LIB, *objs, "-pthread"])
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
