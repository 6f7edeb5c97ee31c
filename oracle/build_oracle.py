"""Build recipe for the CPU oracle (test infrastructure): g++ -> oracle/_build/libgs_oracle.so.

Flags: -ffp-contract=off so every FP32 multiply and add rounds on its own (the evaluation
order the CUDA kernels reproduce with -fmad=false); OpenMP for the CPU-baseline leg.
gs_oracle64.cpp is the FP64 twin used as the precision tier's error reference;
gs_oracle_ply.cpp restates the PLY vertex -> record conversion; gs_oracle_wgpusort.cpp re-executes
the reference's radix sorter workgroup by workgroup (the second sort oracle).
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libgs_oracle.so")
SRCS = [os.path.join(HERE, "gs_oracle.cpp"), os.path.join(HERE, "gs_oracle64.cpp"), os.path.join(HERE, "gs_oracle_ply.cpp"),
        os.path.join(HERE, "gs_oracle_wgpusort.cpp")]


def build(force=False, verbose=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    deps = SRCS + [os.path.join(ROOT, "include", "gs_record.h")]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(d) for d in deps):
        return LIB
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = [
        "g++", "-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
        "-Wall", "-I", os.path.join(ROOT, "include"), *SRCS, "-o", tmp,
    ]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
