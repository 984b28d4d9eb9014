"""Build recipe for the CPU oracle (test infrastructure, never shipped).

Compiles oracle/sflow_oracle.c into oracle/libsflow_oracle.so with gcc,
FP64 with no FMA contraction (-ffp-contract=off) so the operation order of
the restatement is what executes, and OpenMP for the timed CPU baseline.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "sflow_oracle.c")
LIB = os.path.join(HERE, "libsflow_oracle.so")


def build_oracle(force=False, verbose=False):
    deps = [SRC, os.path.join(HERE, "..", "include", "sflow.h"),
            os.path.join(HERE, "..", "imex_sflow2d_dev_gb300", "csrc", "sflow_math.h")]
    if (not force and os.path.exists(LIB)
            and all(os.path.getmtime(LIB) >= os.path.getmtime(d) for d in deps)):
        return LIB
    cmd = ["gcc", "-O2", "-std=gnu11", "-fPIC", "-shared", "-fopenmp",
           "-ffp-contract=off", "-fno-fast-math", "-Wall", "-Wno-unused-function",
           "-o", LIB + ".tmp", SRC, "-lm"]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv, verbose=True))
