"""Build oracle/libns_ref_cpu.so, the C++/OpenMP restatement of the reference
step (test infrastructure and the timed CPU baseline; see ns_ref_cpu.cpp).

Plain g++ on one source file: -O3 -fopenmp, no machine-specific flags, so
the same recipe builds on x86 and Arm hosts."""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "ns_ref_cpu.cpp")
OUT = os.path.join(HERE, "libns_ref_cpu.so")


def build(verbose: bool = False) -> str:
    if not os.path.exists(OUT) or os.path.getmtime(OUT) < os.path.getmtime(SRC):
        cmd = ["g++", "-O3", "-fopenmp", "-std=c++17", "-shared", "-fPIC", "-fcx-limited-range", SRC, "-o", OUT]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(OUT)
    return OUT


if __name__ == "__main__":
    build(verbose=True)
