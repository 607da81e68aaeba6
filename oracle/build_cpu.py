"""Builds the oracle's C restatement (CPU baseline) into oracle/_build/.

Test and benchmark infrastructure only: the library built here is the CPU
restatement of the reference's path that bench.py times as the reference arm;
the product never loads it.
"""

from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "vk_cpu.c")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libvk_cpu.so")


def build(force: bool = False, verbose: bool = False) -> str | None:
    if not os.path.exists(SRC):
        return None
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(
            os.path.getmtime(SRC), os.path.getmtime(os.path.abspath(__file__))):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cmd = ["gcc", "-O3", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-o", LIB + ".tmp", SRC, "-lm", "-ldl"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"gcc failed:\n{r.stdout}\n{r.stderr}")
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
