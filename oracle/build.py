"""Builds the oracle (test infrastructure only) with g++.

  oracle/_build/libmdref.so      serial, -ffp-contract=off: the parity checker
  oracle/_build/libmdref_omp.so  OpenMP, -O2 -ffast-math (the reference's src/Makefile:2 flags):
                                 the CPU baseline timed by bench.py
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build")
SRC = os.path.join(HERE, "mdref.cpp")

VARIANTS = {
    "libmdref.so": ["-O2", "-ffp-contract=off", "-fcx-limited-range"],
    "libmdref_omp.so": ["-O2", "-ffast-math", "-fopenmp"],
}


def _one(name, flags):
    dst = os.path.join(OUT, name)
    if os.path.exists(dst) and os.path.getmtime(dst) >= os.path.getmtime(SRC):
        return dst
    cmd = ["g++", "-std=c++17", "-fPIC", "-shared", *flags, SRC, "-o", dst + ".tmp"]
    subprocess.run(cmd, check=True)
    os.replace(dst + ".tmp", dst)
    return dst


def build():
    os.makedirs(OUT, exist_ok=True)
    with ThreadPoolExecutor(2) as ex:
        return list(ex.map(lambda kv: _one(*kv), VARIANTS.items()))


def path(name="libmdref.so"):
    return os.path.join(OUT, name)


if __name__ == "__main__":
    print(build())
    sys.exit(0)
