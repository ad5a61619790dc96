"""Build recipe of the CPU oracle (test infrastructure only).

Compiles oracle/apic_oracle.cpp, the C++ restatement of the reference step,
into oracle/liboracle.so: -ffp-contract=off and no -ffast-math so float
arithmetic rounds exactly as written; OpenMP for the timed CPU baseline.
The reference itself (Rust) cannot be compiled here: there is no cargo/rustc
and its crates (rdst, wide, ultraviolet, rayon) are not vendored.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "apic_oracle.cpp")
# The benchmark scenes' particle generator (host code, no GPU), compiled in
# under oracle_* names so that the CPU arm generates its inputs without
# loading the GPU library.
SCENE_SRC = os.path.join(os.path.dirname(HERE), "apic-fluid-simulation_gb300", "csrc", "scene.cpp")
SCENE_NAMES = ["-Dapic_scene_count=oracle_scene_count", "-Dapic_scene_fill=oracle_scene_fill"]
LIB = os.path.join(HERE, "liboracle.so")
FLAGS = ["-std=c++20", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC", "-shared"]


def build(force: bool = False) -> str:
    deps = [SRC, SCENE_SRC, os.path.abspath(__file__), os.path.join(HERE, "apic_oracle.h"),
            os.path.join(os.path.dirname(HERE), "include", "apic_gpu.h")]
    if force or not os.path.exists(LIB) or any(os.path.getmtime(d) > os.path.getmtime(LIB) for d in deps):
        cmd = ["g++"] + FLAGS + SCENE_NAMES + ["-o", LIB, SRC, SCENE_SRC]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"oracle build failed: {' '.join(cmd)}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
