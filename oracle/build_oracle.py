"""Builds the CPU oracle (test infrastructure only) into oracle/_build/.

Used by tests/, __graft_entry__ (smoke check and build) and bench.py's CPU
baseline leg. -ffp-contract=off keeps every a*b+c unfused, as in the reference's
broadcasts; OpenMP threads the per-cell loops (results do not depend on the
thread count).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "hymor_oracle.cpp")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libhymor_oracle.so")


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        tmp = LIB + f".{os.getpid()}.tmp"
        cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared",
               "-o", tmp, SRC]
        subprocess.check_call(cmd)
        os.replace(tmp, LIB)
    return LIB


def load() -> ctypes.CDLL:
    return ctypes.CDLL(build())


if __name__ == "__main__":
    print(build(force=True))
